// Host-side string tables for the FCI build (one set per spin).
//
// Everything here is O(D_sigma * excitations) and tiny next to the CRS (for
// L=12, 6 electrons: 924 strings x 262 neighbours). The floating-point parts
// that depend only on one spin string are summed here in exactly the order of
// the reference element functions, so that the device only appends the
// opposite-spin terms and every CRS value comes out bit-identical:
//   get_diag_cont_one_bitstring  (CIMethod.cpp:329-342)  -> diag
//   one_diff_orbital, same-spin part (CIMethod.cpp:409-416) -> s_part
//   two_diff_orbitals(up1,up2)   (CIMethod.cpp:429-442)  -> d_val
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <thread>

#include "cigpu_internal.h"

namespace cigpu {
namespace {

struct Eri {
    const double *e;
    size_t L1, L2, L3;
    // physics <ij|kl> = chemist (ik|jl)  (Hamiltonian.h:45)
    double V(int i, int j, int k, int l) const { return e[i * L3 + k * L2 + j * L1 + l]; }
};

int64_t binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

// Colex rank = sum_m C(p_m, m) over set bits p_1 < p_2 < ... (CIMethod.cpp:732-747);
// bt[p * 65 + m] = C(p, m).
uint32_t rank_of(uint64_t s, const std::vector<int64_t> &bt) {
    int64_t r = 0;
    int m = 0;
    while (s) {
        int p = __builtin_ctzll(s);
        ++m;
        r += bt[p * 65 + m];
        s &= s - 1;
    }
    return static_cast<uint32_t>(r);
}

inline uint64_t next_comb(uint64_t v) {
    uint64_t t = v | (v - 1);
    return (t + 1) | (((~t & -~t) - 1) >> (__builtin_ctzll(v) + 1));
}

// get_nstacked (CIMethod.cpp:382-396): set bits of `common` strictly between the two orbitals.
int nstacked(int a, int b, uint64_t common) {
    int lo = a < b ? a : b, hi = a < b ? b : a;
    uint64_t mask = (hi > lo + 1) ? ((((uint64_t)1 << hi) - 1) & ~(((uint64_t)1 << (lo + 1)) - 1)) : 0;
    return __builtin_popcountll(common & mask);
}

// Stable LSD radix sort of packed entries by their low 32 bits (the target
// rank, < 2^nbits), one byte per pass.
void sort_by_target(std::vector<uint64_t> &a, std::vector<uint64_t> &tmp, int nbits) {
    tmp.resize(a.size());
    for (int shift = 0; shift < nbits; shift += 8) {
        uint32_t cnt[257] = {0};
        for (uint64_t x : a) ++cnt[(((uint32_t)x) >> shift & 255u) + 1];
        for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
        for (uint64_t x : a) tmp[cnt[((uint32_t)x) >> shift & 255u]++] = x;
        a.swap(tmp);
    }
}

}  // namespace

void build_spin_tables(int L, int n, const double *h, const double *eri, SpinTables &t) {
    if (L < 1 || L > kMaxL || n < 0 || n > L) throw std::invalid_argument("spin table size");
    Eri E{eri, (size_t)L, (size_t)L * L, (size_t)L * L * L};
    t.L = L;
    t.n = n;
    t.D = binom(L, n);
    t.ns = n * (L - n);
    t.nd = (int)(binom(n, 2) * binom(L - n, 2));
    t.nfull = 1 + t.ns + t.nd;
    t.nsing = 1 + t.ns;
    const int64_t D = t.D;
    t.strings.resize(D);
    t.occ.assign(D * (size_t)std::max(n, 1), 0);
    t.diag.resize(D);
    t.s_target.resize(D * (size_t)t.ns);
    t.s_part.resize(D * (size_t)t.ns);
    t.s_info.resize(D * (size_t)t.ns);
    t.d_target.resize(D * (size_t)t.nd);
    t.d_val.resize(D * (size_t)t.nd);
    t.d_hi.resize(D * (size_t)t.nd);
    t.d_lo.resize(D * (size_t)t.nd);
    t.nb_full.resize(D * (size_t)t.nfull);
    t.nb_sing.resize(D * (size_t)t.nsing);

    uint64_t s = n == 0 ? 0 : (n >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << n) - 1));
    for (int64_t I = 0; I < D; ++I) {
        t.strings[I] = s;
        if (n > 0 && I + 1 < D) s = next_comb(s);
    }

    std::vector<int64_t> bt(65 * 65, 0);
    for (int p = 0; p <= 64; ++p)
        for (int m = 0; m <= 64 && m <= p; ++m) bt[p * 65 + m] = (p <= 62) ? binom(p, m) : 0;
    auto work = [&](int64_t I0, int64_t I1) {
    std::vector<uint64_t> full, sing, tmp;
    int nbits = 1;
    while (nbits < 32 && ((int64_t)1 << nbits) < D) ++nbits;
    for (int64_t I = I0; I < I1; ++I) {
        const uint64_t si = t.strings[I];
        int o[64], k = 0, v[64], kv = 0;
        for (int b = 0; b < L; ++b) {
            if (si >> b & 1)
                o[k++] = b;
            else
                v[kv++] = b;
        }
        for (int a = 0; a < n; ++a) t.occ[I * n + a] = (uint8_t)o[a];
        // diagonal part of one string, reference order
        double d = 0;
        for (int a = 0; a < n; ++a) d += h[o[a] * L + o[a]];
        for (int a = 0; a < n - 1; ++a)
            for (int b = a + 1; b < n; ++b) d += E.V(o[a], o[b], o[a], o[b]) - E.V(o[a], o[b], o[b], o[a]);
        t.diag[I] = d;

        full.clear();
        sing.clear();
        full.push_back((uint64_t)I | ((uint64_t)kSelf << 32));
        sing.push_back((uint64_t)I | ((uint64_t)kSelf << 32));
        // singles: row orbital j (occupied) -> col orbital l (empty)
        int si_idx = 0;
        for (int ja = 0; ja < k; ++ja) {
            const int j = o[ja];
            for (int la = 0; la < kv; ++la) {
                const int l = v[la];
                const uint64_t sj = si ^ ((uint64_t)1 << j) ^ ((uint64_t)1 << l);
                const uint32_t J = rank_of(sj, bt);
                const int lo = j < l ? j : l, hi = j < l ? l : j;
                const uint64_t common = si & sj;
                // one_diff_orbital: elemu = T(lo,hi) + sum_z (V(lo,z,hi,z) - V(lo,z,z,hi))
                double e = h[lo * L + hi];
                for (int za = 0; za < k; ++za) {  // common orbitals ascending: occupied minus j
                    const int z = o[za];
                    if (z == j) continue;
                    e += E.V(lo, z, hi, z) - E.V(lo, z, z, hi);
                }
                const int odd = nstacked(lo, hi, common) & 1;
                const size_t at = (size_t)I * t.ns + si_idx;
                t.s_target[at] = J;
                t.s_part[at] = e;
                t.s_info[at] = (uint32_t)lo | (uint32_t)hi << 6 | (uint32_t)j << 12 | (uint32_t)l << 18 |
                               (uint32_t)odd << 24;
                full.push_back((uint64_t)J | ((uint64_t)kSingle << 32) | ((uint64_t)si_idx << 34));
                sing.push_back((uint64_t)J | ((uint64_t)kSingle << 32) | ((uint64_t)si_idx << 34));
                ++si_idx;
            }
        }
        // same-spin doubles j1<j2 occupied -> l1<l2 empty
        int di = 0;
        for (int a1 = 0; a1 < k; ++a1) {
            const int j1 = o[a1];
            for (int a2 = a1 + 1; a2 < k; ++a2) {
                const int j2 = o[a2];
                for (int b1 = 0; b1 < kv; ++b1) {
                    const int l1 = v[b1];
                    for (int b2 = b1 + 1; b2 < kv; ++b2) {
                        const int l2 = v[b2];
                        const uint64_t sj =
                            si ^ ((uint64_t)1 << j1) ^ ((uint64_t)1 << j2) ^ ((uint64_t)1 << l1) ^ ((uint64_t)1 << l2);
                        const uint32_t J = rank_of(sj, bt);
                        // the reference evaluates the upper element: row = the lower-ranked string
                        const uint64_t row = (J > (uint32_t)I) ? si : sj;
                        const uint64_t colS = (J > (uint32_t)I) ? sj : si;
                        const uint64_t common = si & sj;
                        int a[4], na = 0, nb = 2;
                        // arrange_order (CIMethod.cpp:353-380): row orbitals first, ascending
                        for (uint64_t x = row ^ colS; x; x &= x - 1) {
                            const int b = __builtin_ctzll(x);
                            if (row >> b & 1)
                                a[na++] = b;
                            else
                                a[nb++] = b;
                        }
                        (void)colS;
                        const int diff = nstacked(a[0], a[1], common) + nstacked(a[2], a[3], common);
                        double e = E.V(a[0], a[1], a[2], a[3]) - E.V(a[0], a[1], a[3], a[2]);
                        if (diff % 2 != 0) e *= -1;
                        const size_t at = (size_t)I * t.nd + di;
                        t.d_target[at] = J;
                        t.d_val[at] = e;
                        split_fp32(e, t.d_hi[at], t.d_lo[at]);
                        full.push_back((uint64_t)J | ((uint64_t)kDouble << 32) | ((uint64_t)di << 34));
                        ++di;
                    }
                }
            }
        }
        sort_by_target(full, tmp, nbits);
        sort_by_target(sing, tmp, nbits);
        std::memcpy(&t.nb_full[(size_t)I * t.nfull], full.data(), full.size() * sizeof(uint64_t));
        std::memcpy(&t.nb_sing[(size_t)I * t.nsing], sing.data(), sing.size() * sizeof(uint64_t));
    }
    };
    // strings are independent: split them over host threads (disjoint output ranges)
    const int64_t nt = std::max<int64_t>(1, std::min<int64_t>((int64_t)std::thread::hardware_concurrency(), D / 64));
    if (nt <= 1) {
        work(0, D);
    } else {
        std::vector<std::thread> th;
        for (int64_t q = 0; q < nt; ++q) th.emplace_back(work, D * q / nt, D * (q + 1) / nt);
        for (auto &x : th) x.join();
    }
}

}  // namespace cigpu
