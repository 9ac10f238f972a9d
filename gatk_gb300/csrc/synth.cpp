// synth.cpp -- deterministic synthetic active-region generator for the PairHMM workloads.
//
// Every region is generated from its own xoshiro256** stream seeded from (seed, region index),
// so any region range can be generated on its own (streaming) and in parallel, and the bytes are
// identical on x86_64 and aarch64: only IEEE basic operations and sqrt are used (no libm
// transcendental; ln/exp are evaluated below by series), and the file is compiled with
// -ffp-contract=off.
//
// Workloads (seed in parentheses):
//   0 (0) one region: 8 haplotypes (a uniform-ACGT base haplotype of 300 bp plus 7 variants with
//         1-3 SNPs or one 1-10 bp indel), 64 reads of 150 bp from a uniform haplotype at a uniform
//         offset, 1% substitutions, 0.1% indels, base Q ~ U[10,40], ins/del Q 45, GCP 10.
//   1 (1) 10,000 regions: haplotype count U[2,32], base length U[200,600]; reads per region
//         lognormal(4,1) rounded and clipped to [1,1000]; read length U[100,250]; as workload 0.
//   2 (2) 2,000 long-pair regions: haplotypes U[4,16] of length U[1500,3000]; reads U[8,64] of
//         length U[800,2000]; 5% substitutions, 1% indels; base Q U[5,25]; ins/del Q U[20,45].
//   3 (3) 512 short-tandem-repeat regions x 8 reads (4,096 pairs): one 300 bp haplotype with an
//         STR of period 1-8 and 2-20 repeats centred in random flanks; 150 bp reads with
//         whole-unit indel errors at 0.5% x period inside the repeat tract.
//   4 (4) workload 1's distributions over 100,000 regions, plus a 5% tail of high-depth
//         regions with 2,000 reads x 64 haplotypes.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ghmm_synth.h"

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    Rng(uint64_t seed, uint64_t stream) {
        uint64_t x = seed * 0x2545F4914F6CDD1DULL + stream * 0x9E3779B97F4A7C15ULL + 0x1234567ULL;
        for (auto &v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform integer in [lo, hi]
    int64_t uniform(int64_t lo, int64_t hi) {
        const uint64_t span = (uint64_t)(hi - lo) + 1;
        return lo + (int64_t)((unsigned __int128)next() * span >> 64);
    }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ln(x), x > 0: exact binary exponent split plus an atanh series on the mantissa.
double det_log(double x) {
    int e = 0;
    double m = x;
    while (m >= 2.0) { m *= 0.5; e++; }
    while (m < 1.0) { m *= 2.0; e--; }
    if (m > 1.4142135623730951) { m *= 0.5; e++; }
    const double t = (m - 1.0) / (m + 1.0), t2 = t * t;
    double term = t, sum = 0.0;
    for (int k = 1; k < 60; k += 2) {
        sum += term / (double)k;
        term *= t2;
    }
    return 2.0 * sum + (double)e * 0.6931471805599453;
}

// exp(x) for |x| < 700: reduce by ln2, Taylor on the remainder, scale by 2^k.
double det_exp(double x) {
    const double ln2 = 0.6931471805599453;
    double kf = x / ln2;
    long k = (long)(kf >= 0 ? kf + 0.5 : kf - 0.5);
    const double r = x - (double)k * ln2;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 30; n++) {
        term *= r / (double)n;
        sum += term;
    }
    while (k > 0) { sum *= 2.0; k--; }
    while (k < 0) { sum *= 0.5; k++; }
    return sum;
}

// standard normal by the Marsaglia polar method
double normal(Rng &g) {
    for (;;) {
        const double u = 2.0 * g.unit() - 1.0, v = 2.0 * g.unit() - 1.0;
        const double s = u * u + v * v;
        if (s > 0.0 && s < 1.0) return u * __builtin_sqrt(-2.0 * det_log(s) / s);
    }
}

const char kBases[4] = {'A', 'C', 'G', 'T'};

char random_base(Rng &g) { return kBases[g.uniform(0, 3)]; }
char other_base(Rng &g, char b) {
    for (;;) {
        const char c = random_base(g);
        if (c != b) return c;
    }
}

struct RegionOut {
    std::vector<int32_t> hap_len, read_len;
    std::vector<uint8_t> hap_bases;
    std::vector<uint8_t> bases, quals, ins, dels, gcp;
};

struct ReadModel {
    double p_sub, p_indel;
    int bq_lo, bq_hi;
    int iq_lo, iq_hi;  // ins/del quality range (equal bounds = constant)
    int gcp;
};

// Variant haplotype: 1-3 SNPs or one 1-10 bp insertion/deletion (50/50).
std::string make_variant(Rng &g, const std::string &base) {
    std::string h = base;
    if (g.uniform(0, 1) == 0) {
        const int n = (int)g.uniform(1, 3);
        for (int k = 0; k < n; k++) {
            const size_t pos = (size_t)g.uniform(0, (int64_t)h.size() - 1);
            h[pos] = other_base(g, h[pos]);
        }
    } else {
        const int len = (int)g.uniform(1, 10);
        const size_t pos = (size_t)g.uniform(1, (int64_t)h.size() - 2);
        if (g.uniform(0, 1) == 0) {
            std::string ins;
            for (int k = 0; k < len; k++) ins.push_back(random_base(g));
            h.insert(pos, ins);
        } else {
            const size_t l = std::min((size_t)len, h.size() - pos - 1);
            h.erase(pos, l);
        }
    }
    return h;
}

void emit_quals(Rng &g, const ReadModel &m, int R, RegionOut &o) {
    for (int i = 0; i < R; i++) {
        o.quals.push_back((uint8_t)g.uniform(m.bq_lo, m.bq_hi));
        o.ins.push_back((uint8_t)g.uniform(m.iq_lo, m.iq_hi));
        o.dels.push_back((uint8_t)g.uniform(m.iq_lo, m.iq_hi));
        o.gcp.push_back((uint8_t)m.gcp);
    }
}

// A read of length R sampled from haplotype h at a uniform offset with sequencing errors.
// Past the end of the haplotype the read continues with random bases.
void sample_read(Rng &g, const std::string &h, int R, const ReadModel &m, RegionOut &o) {
    const int64_t H = (int64_t)h.size();
    size_t pos = (size_t)(H > R ? g.uniform(0, H - R) : 0);
    int produced = 0;
    while (produced < R) {
        const char t = pos < h.size() ? h[pos] : random_base(g);
        const double u = g.unit();
        if (u < m.p_indel * 0.5) {  // insertion of a random base before the template base
            o.bases.push_back((uint8_t)random_base(g));
            produced++;
            continue;
        } else if (u < m.p_indel) {  // deletion: skip the template base
            pos++;
            continue;
        }
        char b = t;
        if (g.unit() < m.p_sub) b = other_base(g, t);
        o.bases.push_back((uint8_t)b);
        produced++;
        pos++;
    }
    o.read_len.push_back(R);
    emit_quals(g, m, R, o);
}

void push_hap(const std::string &h, RegionOut &o) {
    o.hap_len.push_back((int32_t)h.size());
    o.hap_bases.insert(o.hap_bases.end(), h.begin(), h.end());
}

void gen_standard_region(Rng &g, int n_haps, int base_len, int n_reads, int rl_lo, int rl_hi, const ReadModel &m,
                         RegionOut &o) {
    std::string base;
    for (int i = 0; i < base_len; i++) base.push_back(random_base(g));
    std::vector<std::string> haps{base};
    for (int a = 1; a < n_haps; a++) haps.push_back(make_variant(g, base));
    for (auto &h : haps) push_hap(h, o);
    for (int r = 0; r < n_reads; r++) {
        const int R = (int)g.uniform(rl_lo, rl_hi);
        const std::string &h = haps[(size_t)g.uniform(0, n_haps - 1)];
        sample_read(g, h, R, m, o);
    }
}

int lognormal_reads(Rng &g, double mu, double sigma, int lo, int hi) {
    const double v = det_exp(mu + sigma * normal(g));
    long n = (long)(v + 0.5);
    if (n < lo) n = lo;
    if (n > hi) n = hi;
    return (int)n;
}

void gen_str_region(Rng &g, RegionOut &o) {
    const int period = (int)g.uniform(1, 8), repeats = (int)g.uniform(2, 20);
    std::string unit;
    for (int i = 0; i < period; i++) unit.push_back(random_base(g));
    std::string tract;
    for (int i = 0; i < repeats; i++) tract += unit;
    const int H = 300;
    const int left = (H - (int)tract.size()) / 2;
    std::string h;
    for (int i = 0; i < left; i++) h.push_back(random_base(g));
    const size_t t0 = h.size();
    h += tract;
    const size_t t1 = h.size();
    while ((int)h.size() < H) h.push_back(random_base(g));
    push_hap(h, o);
    const ReadModel m{0.01, 0.001, 10, 40, 45, 45, 10};
    const double p_unit_indel = 0.005 * period;
    for (int r = 0; r < 8; r++) {
        const int R = 150;
        size_t pos = (size_t)g.uniform(0, H - R);
        int produced = 0;
        while (produced < R) {
            const bool in_tract = pos >= t0 && pos < t1;
            const char t = pos < h.size() ? h[pos] : random_base(g);
            if (in_tract && (pos - t0) % (size_t)period == 0 && g.unit() < p_unit_indel) {
                if (g.uniform(0, 1) == 0) {  // one extra repeat unit
                    for (int k = 0; k < period && produced < R; k++, produced++) o.bases.push_back((uint8_t)unit[k]);
                } else {  // one repeat unit missing
                    pos += (size_t)period;
                }
                continue;
            }
            const double u = g.unit();
            if (!in_tract && u < m.p_indel * 0.5) {
                o.bases.push_back((uint8_t)random_base(g));
                produced++;
                continue;
            } else if (!in_tract && u < m.p_indel) {
                pos++;
                continue;
            }
            char b = t;
            if (g.unit() < m.p_sub) b = other_base(g, t);
            o.bases.push_back((uint8_t)b);
            produced++;
            pos++;
        }
        o.read_len.push_back(R);
        emit_quals(g, m, R, o);
    }
}

void gen_region(int workload, uint64_t seed, int64_t region, RegionOut &o) {
    Rng g(seed, (uint64_t)region);
    switch (workload) {
        case 0: {
            const ReadModel m{0.01, 0.001, 10, 40, 45, 45, 10};
            gen_standard_region(g, 8, 300, 64, 150, 150, m, o);
            break;
        }
        case 1: {
            const ReadModel m{0.01, 0.001, 10, 40, 45, 45, 10};
            const int nh = (int)g.uniform(2, 32), bl = (int)g.uniform(200, 600);
            const int nr = lognormal_reads(g, 4.0, 1.0, 1, 1000);
            gen_standard_region(g, nh, bl, nr, 100, 250, m, o);
            break;
        }
        case 2: {
            const ReadModel m{0.05, 0.01, 5, 25, 20, 45, 10};
            const int nh = (int)g.uniform(4, 16), bl = (int)g.uniform(1500, 3000);
            const int nr = (int)g.uniform(8, 64);
            gen_standard_region(g, nh, bl, nr, 800, 2000, m, o);
            break;
        }
        case 3:
            gen_str_region(g, o);
            break;
        case 4: {
            const ReadModel m{0.01, 0.001, 10, 40, 45, 45, 10};
            if (g.unit() < 0.05) {
                const int bl = (int)g.uniform(200, 600);
                gen_standard_region(g, 64, bl, 2000, 100, 250, m, o);
            } else {
                const int nh = (int)g.uniform(2, 32), bl = (int)g.uniform(200, 600);
                const int nr = lognormal_reads(g, 4.0, 1.0, 1, 1000);
                gen_standard_region(g, nh, bl, nr, 100, 250, m, o);
            }
            break;
        }
        default:
            break;
    }
}

}  // namespace

struct ghmm_synth {
    std::vector<int64_t> region_read_off, region_hap_off, read_off, hap_off, out_off;
    std::vector<uint8_t> bases, quals, ins, dels, gcp, hap_bases;
};

extern "C" int64_t ghmm_synth_default_regions(int32_t workload) {
    switch (workload) {
        case 0: return 1;
        case 1: return 10000;
        case 2: return 2000;
        case 3: return 512;
        case 4: return 100000;
        default: return -1;
    }
}

extern "C" int ghmm_synth_generate(int32_t workload, uint64_t seed, int64_t region_begin, int64_t region_end,
                                   int32_t threads, ghmm_synth **out) {
    if (!out || workload < 0 || workload > 4 || region_begin < 0 || region_end < region_begin) return 1;
    const int64_t n = region_end - region_begin;
    std::vector<RegionOut> regs((size_t)n);
    int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = (int)std::min<int64_t>(nt, std::max<int64_t>(1, n));
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
        pool.emplace_back([&, t] {
            for (int64_t i = t; i < n; i += nt) gen_region(workload, seed, region_begin + i, regs[(size_t)i]);
        });
    for (auto &th : pool) th.join();

    auto *s = new ghmm_synth();
    int64_t nreads = 0, nhaps = 0, rbytes = 0, hbytes = 0;
    for (auto &r : regs) {
        nreads += (int64_t)r.read_len.size();
        nhaps += (int64_t)r.hap_len.size();
        rbytes += (int64_t)r.bases.size();
        hbytes += (int64_t)r.hap_bases.size();
    }
    s->region_read_off.reserve((size_t)n + 1);
    s->region_hap_off.reserve((size_t)n + 1);
    s->out_off.reserve((size_t)n + 1);
    s->read_off.reserve((size_t)nreads + 1);
    s->hap_off.reserve((size_t)nhaps + 1);
    for (auto *v : {&s->bases, &s->quals, &s->ins, &s->dels, &s->gcp}) v->reserve((size_t)rbytes);
    s->hap_bases.reserve((size_t)hbytes);
    s->region_read_off.push_back(0);
    s->region_hap_off.push_back(0);
    s->out_off.push_back(0);
    s->read_off.push_back(0);
    s->hap_off.push_back(0);
    for (auto &r : regs) {
        for (int32_t L : r.read_len) s->read_off.push_back(s->read_off.back() + L);
        for (int32_t L : r.hap_len) s->hap_off.push_back(s->hap_off.back() + L);
        s->region_read_off.push_back(s->region_read_off.back() + (int64_t)r.read_len.size());
        s->region_hap_off.push_back(s->region_hap_off.back() + (int64_t)r.hap_len.size());
        s->out_off.push_back(s->out_off.back() + (int64_t)r.read_len.size() * (int64_t)r.hap_len.size());
        s->bases.insert(s->bases.end(), r.bases.begin(), r.bases.end());
        s->quals.insert(s->quals.end(), r.quals.begin(), r.quals.end());
        s->ins.insert(s->ins.end(), r.ins.begin(), r.ins.end());
        s->dels.insert(s->dels.end(), r.dels.begin(), r.dels.end());
        s->gcp.insert(s->gcp.end(), r.gcp.begin(), r.gcp.end());
        s->hap_bases.insert(s->hap_bases.end(), r.hap_bases.begin(), r.hap_bases.end());
        r = RegionOut();
    }
    *out = s;
    return 0;
}

extern "C" int ghmm_synth_view(const ghmm_synth *s, ghmm_synth_arrays *a) {
    if (!s || !a) return 1;
    a->n_regions = (int64_t)s->region_read_off.size() - 1;
    a->n_reads = (int64_t)s->read_off.size() - 1;
    a->n_haps = (int64_t)s->hap_off.size() - 1;
    a->read_bytes = (int64_t)s->bases.size();
    a->hap_bytes = (int64_t)s->hap_bases.size();
    a->n_out = s->out_off.back();
    a->region_read_off = s->region_read_off.data();
    a->region_hap_off = s->region_hap_off.data();
    a->read_off = s->read_off.data();
    a->hap_off = s->hap_off.data();
    a->out_off = s->out_off.data();
    a->bases = s->bases.data();
    a->quals = s->quals.data();
    a->ins = s->ins.data();
    a->dels = s->dels.data();
    a->gcp = s->gcp.data();
    a->hap_bases = s->hap_bases.data();
    return 0;
}

extern "C" void ghmm_synth_free(ghmm_synth *s) { delete s; }
