// 1- and 2-RDMs of a CI vector on the device.
//
// Replaces CIDens::construct_density with DensFCI / DensDOCI (CIDens.cpp:323-334,
// 1073-1224, 1530-1631). The reference loops over all determinant pairs and
// classifies each by popcount (O(dim^2)); here only connected pairs contribute and
// every sum has a fixed order (no atomics, bit-reproducible).
//
// FCI. Write C[Ia][Ib] for the CI vector. Every contribution of fill_density_matrix
// (CIDens.cpp:676-881) with a pair (I, J), I <= J in row order, is one of
//   * alpha pair (Ia, Ja >= Ia, same Ib): diagonal, single or alpha-alpha double.
//     Its weight only needs the string-pair densities
//        Da0[Ia,Ja]    = sum_b C[Ia][b] C[Ja][b]
//        Daz[Ia,Ja][z] = sum_b C[Ia][b] C[Ja][b] n_z(b)    (beta spectators z)
//   * beta pair (Ib, Jb > Ib, same Ia): the mirror image with C transposed;
//   * alpha-beta double (Ia -> Ja = Ia - ar + ac, ac > ar; Ib -> Jb = Ib - br + bc):
//        Gamma_ab[(ar,br),(ac,bc)] += s_a s_b C[Ia][Ib] C[Ja][Jb].
// Step 1 computes the pair densities (one warp per string pair). Step 2 sums, for
// each RDM element, a host-built list of (density, +/-1) terms -- the list encodes
// the reference's orbital ordering and antisymmetry signs (add_one_rdm /
// add_two_rdm, CIDens.cpp:227-292). Step 3 handles the alpha-beta doubles: one
// block per alpha excitation (ar, ac) (split in a few parts), one thread per beta
// excitation type (br, bc), looping over the strings that admit it.
//
// DOCI: one block of L*L threads per slice of pair strings; thread (j, k)
// accumulates c_I^2 n_j n_k and the pair-hop products c_I c_J (DensDOCI,
// CIDens.cpp:1073-1224).
//
// Storage follows CIDens: the 1-RDM and each 2-RDM block are symmetric pair
// matrices (Vector2d, matrix.cpp:674-690), accumulated on (min, max) and mirrored.
//
// Determinant lists (DensFILE) are handled in dets.cu: a pair scan with 64-bit
// fixed-point integer atomics (order-independent sums, also bit-reproducible).
#include <algorithm>
#include <memory>
#include <mutex>
#include <stdexcept>

#include "checked.cuh"
#include "crs.cuh"

namespace cigpu {
namespace {

constexpr int kRdmThreads = 256;

inline int pidx(int p, int q, int L) { return p * L + q - (p + 1) * (p + 2) / 2; }

// C(n, k) for n, k < 64 (strings of up to 63 orbitals), filled once.
struct BinomTable {
    int64_t c[64][65];
    BinomTable() {
        for (int n = 0; n < 64; ++n)
            for (int k = 0; k <= 64; ++k) c[n][k] = d_binom(n, k);
    }
};

uint32_t hrank(uint64_t s) {
    static const BinomTable bt;
    int64_t r = 0;
    int m = 0;
    while (s) {
        ++m;
        r += bt.c[__builtin_ctzll(s)][m];
        s &= s - 1;
    }
    return (uint32_t)r;
}

int hnstacked(int a, int b, uint64_t common) {
    const int lo = std::min(a, b), hi = std::max(a, b);
    int c = 0;
    for (int i = lo + 1; i < hi; ++i) c += (int)((common >> i) & 1);
    return c;
}

// One spin's pair list and its RDM terms.
struct PairPlan {
    std::vector<uint32_t> I, J;  // pairs: [self..., singles..., doubles...]
    int nz = 0;                  // the first nz pairs (self + singles) also need Dz
};

struct Plan {
    int L, np;
    int64_t Da, Db;
    PairPlan a, b;
    size_t off_ga, off_gb, off_g0, off_g1, off_g2, nslots;
    // density layout: [Da0 | Daz | Db0 | Dbz]
    size_t off_da0, off_daz, off_db0, off_dbz, ndens;
    struct Term {
        uint32_t slot, dens;
        int8_t coef;
    };
    std::vector<Term> terms;  // in generation order; grouped by slot (stably) afterwards
    // alpha-beta doubles
    std::vector<uint32_t> ap_ptr;   // [np+1] alpha pairs per (ar<ac)
    std::vector<uint64_t> ap;       // Ia | Ja << 32
    std::vector<int8_t> ap_sign;
    std::vector<uint32_t> bx_ptr;   // [L*L+1] beta excitations per (br, bc)
    std::vector<uint64_t> bx;       // Ib | Jb << 32
    std::vector<int8_t> bx_sign;
};

void add_term(Plan &P, size_t slot, size_t dens, int coef) {
    P.terms.push_back({(uint32_t)slot, (uint32_t)dens, (int8_t)coef});
}

// Slot of a symmetric pair matrix entry (min, max) of dimension dimx at offset off.
size_t sym_slot(size_t off, size_t dimx, size_t A, size_t B) {
    return off + std::min(A, B) * dimx + std::max(A, B);
}

// add_two_rdm for a same-spin block (CIDens.cpp:240-255): sorts both pairs with sign flips.
void add_two_same(Plan &P, size_t off, int o1, int o2, int o3, int o4, size_t dens, int coef) {
    if (o1 == o2 || o3 == o4) return;
    if (o1 > o2) { std::swap(o1, o2); coef = -coef; }
    if (o3 > o4) { std::swap(o3, o4); coef = -coef; }
    add_term(P, sym_slot(off, P.np, pidx(o1, o2, P.L), pidx(o3, o4, P.L)), dens, coef);
}

void add_two_ab(Plan &P, int o1, int o2, int o3, int o4, size_t dens, int coef) {
    const size_t L = P.L;
    add_term(P, sym_slot(P.off_g1, L * L, o1 * L + o2, o3 * L + o4), dens, coef);
}

// Pairs and terms of one spin. `alpha` selects which 1-RDM / same-spin block and
// where the opposite-spin spectators go in Gamma_ab.
void plan_spin(Plan &P, const SpinTables &t, bool alpha) {
    const int L = P.L, n = t.n;
    PairPlan &pp = alpha ? P.a : P.b;
    const int64_t D = t.D;
    // self pairs
    for (int64_t I = 0; I < D; ++I) {
        pp.I.push_back((uint32_t)I);
        pp.J.push_back((uint32_t)I);
    }
    // upper singles
    struct Single { uint32_t I, J; int lo, hi, sign; uint64_t common; };
    std::vector<Single> singles;
    for (int64_t I = 0; I < D; ++I) {
        const uint64_t s = t.strings[I];
        for (int j = 0; j < L; ++j) {
            if (!((s >> j) & 1)) continue;
            for (int l = j + 1; l < L; ++l) {
                if ((s >> l) & 1) continue;
                const uint64_t u = s ^ ((uint64_t)1 << j) ^ ((uint64_t)1 << l);
                const uint32_t J = hrank(u);  // > I since l > j
                singles.push_back({(uint32_t)I, J, j, l, (hnstacked(j, l, s & u) & 1) ? -1 : 1, s & u});
            }
        }
    }
    for (auto &x : singles) {
        pp.I.push_back(x.I);
        pp.J.push_back(x.J);
    }
    pp.nz = (int)pp.I.size();
    // upper same-spin doubles
    struct Dbl { uint32_t I, J; int o[4]; int sign; };
    std::vector<Dbl> dbls;
    for (int64_t I = 0; I < D; ++I) {
        const uint64_t s = t.strings[I];
        for (int j1 = 0; j1 < L; ++j1) {
            if (!((s >> j1) & 1)) continue;
            for (int j2 = j1 + 1; j2 < L; ++j2) {
                if (!((s >> j2) & 1)) continue;
                for (int l1 = 0; l1 < L; ++l1) {
                    if ((s >> l1) & 1) continue;
                    for (int l2 = l1 + 1; l2 < L; ++l2) {
                        if ((s >> l2) & 1) continue;
                        const uint64_t u = s ^ ((uint64_t)1 << j1) ^ ((uint64_t)1 << j2) ^ ((uint64_t)1 << l1) ^
                                           ((uint64_t)1 << l2);
                        const uint32_t J = hrank(u);
                        if (J <= (uint32_t)I) continue;
                        // fill_two_dense (CIDens.cpp:756-779): row orbitals first, ascending
                        const uint64_t c = s & u;
                        const int diff = hnstacked(j1, j2, c) + hnstacked(l1, l2, c);
                        dbls.push_back({(uint32_t)I, J, {j1, j2, l1, l2}, (diff & 1) ? -1 : 1});
                    }
                }
            }
        }
    }
    for (auto &x : dbls) {
        pp.I.push_back(x.I);
        pp.J.push_back(x.J);
    }
    (void)n;
    // terms
    const size_t d0 = alpha ? P.off_da0 : P.off_db0;
    const size_t dz = alpha ? P.off_daz : P.off_dbz;
    const size_t g1 = alpha ? P.off_ga : P.off_gb;
    const size_t gs = alpha ? P.off_g0 : P.off_g2;
    for (int64_t I = 0; I < D; ++I) {  // self pairs (fill_diagonal, CIDens.cpp:808-853)
        const uint64_t s = t.strings[I];
        int o[64], k = 0;
        for (int b = 0; b < L; ++b)
            if ((s >> b) & 1) o[k++] = b;
        for (int i = 0; i < k; ++i) add_term(P, sym_slot(g1, L, o[i], o[i]), d0 + I, 1);
        for (int i = 0; i < k; ++i)
            for (int j = i + 1; j < k; ++j) add_two_same(P, gs, o[i], o[j], o[i], o[j], d0 + I, 1);
        if (alpha)  // mixed diagonal part, once (alpha side): Gamma_ab(u z, u z) += sum c^2 n_u n_z
            for (int i = 0; i < k; ++i)
                for (int z = 0; z < L; ++z) add_two_ab(P, o[i], z, o[i], z, dz + (size_t)I * L + z, 1);
    }
    for (size_t q = 0; q < singles.size(); ++q) {  // fill_one_dense (CIDens.cpp:676-754)
        const Single &x = singles[q];
        const size_t pi = (size_t)D + q;
        add_term(P, sym_slot(g1, L, x.lo, x.hi), d0 + pi, x.sign);
        for (int z = 0; z < L; ++z) {
            if ((x.common >> z) & 1) add_two_same(P, gs, x.lo, z, x.hi, z, d0 + pi, x.sign);
            if (alpha)
                add_two_ab(P, x.lo, z, x.hi, z, dz + pi * L + z, x.sign);
            else
                add_two_ab(P, z, x.lo, z, x.hi, dz + pi * L + z, x.sign);
        }
    }
    for (size_t q = 0; q < dbls.size(); ++q) {
        const Dbl &x = dbls[q];
        const size_t pi = (size_t)D + singles.size() + q;
        add_two_same(P, gs, x.o[0], x.o[1], x.o[2], x.o[3], d0 + pi, x.sign);
    }
}

void plan_ab(Plan &P, const SpinTables &ta, const SpinTables &tb) {
    const int L = P.L;
    // alpha excitations ar -> ac with ac > ar (the row is the lower-ranked string)
    std::vector<std::vector<std::pair<uint64_t, int8_t>>> apl(P.np);
    for (int64_t I = 0; I < ta.D; ++I) {
        const uint64_t s = ta.strings[I];
        for (int ar = 0; ar < L; ++ar) {
            if (!((s >> ar) & 1)) continue;
            for (int ac = ar + 1; ac < L; ++ac) {
                if ((s >> ac) & 1) continue;
                const uint64_t u = s ^ ((uint64_t)1 << ar) ^ ((uint64_t)1 << ac);
                const int sign = (hnstacked(ar, ac, s & u) & 1) ? -1 : 1;
                apl[pidx(ar, ac, L)].push_back({(uint64_t)I | ((uint64_t)hrank(u) << 32), (int8_t)sign});
            }
        }
    }
    P.ap_ptr.assign(P.np + 1, 0);
    for (int q = 0; q < P.np; ++q) {
        P.ap_ptr[q + 1] = P.ap_ptr[q] + (uint32_t)apl[q].size();
        for (auto &e : apl[q]) {
            P.ap.push_back(e.first);
            P.ap_sign.push_back(e.second);
        }
    }
    // beta excitations br -> bc (any order)
    std::vector<std::vector<std::pair<uint64_t, int8_t>>> bxl((size_t)L * L);
    for (int64_t I = 0; I < tb.D; ++I) {
        const uint64_t s = tb.strings[I];
        for (int br = 0; br < L; ++br) {
            if (!((s >> br) & 1)) continue;
            for (int bc = 0; bc < L; ++bc) {
                if ((s >> bc) & 1) continue;
                const uint64_t u = s ^ ((uint64_t)1 << br) ^ ((uint64_t)1 << bc);
                const int sign = (hnstacked(br, bc, s & u) & 1) ? -1 : 1;
                bxl[(size_t)br * L + bc].push_back({(uint64_t)I | ((uint64_t)hrank(u) << 32), (int8_t)sign});
            }
        }
    }
    P.bx_ptr.assign((size_t)L * L + 1, 0);
    for (size_t q = 0; q < (size_t)L * L; ++q) {
        P.bx_ptr[q + 1] = P.bx_ptr[q] + (uint32_t)bxl[q].size();
        for (auto &e : bxl[q]) {
            P.bx.push_back(e.first);
            P.bx_sign.push_back(e.second);
        }
    }
}

// ---------------------------------------------------------------------------
// Step 1: pair densities. C is D1 x D2 row-major; other = strings of the D2 spin.
__global__ void k_pair_dens(const double *__restrict__ C, int64_t D2, const uint32_t *__restrict__ pI,
                            const uint32_t *__restrict__ pJ, int64_t npairs, int64_t nz,
                            const uint64_t *__restrict__ other, int L, double *__restrict__ d0,
                            double *__restrict__ dz, int64_t D1, unsigned long long *err) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = wid; p < npairs; p += nw) {
        const uint32_t I = pI[p], J = pJ[p];
        if (!CIGPU_CHECK(err, index_ok(I, (uint64_t)D1) && index_ok(J, (uint64_t)D1), kCheckRdmPair, p)) {
            if (lane == 0) d0[p] = 0;  // the same for the whole warp
            if (p < nz)
                for (int z = lane; z < L; z += 32) dz[p * L + z] = 0;
            continue;
        }
        const double *ri = C + (int64_t)I * D2;
        const double *rj = C + (int64_t)J * D2;
        double acc = 0;
        for (int64_t b = lane; b < D2; b += 32) acc += ri[b] * rj[b];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) d0[p] = acc;
        if (p < nz) {
            for (int z0 = 0; z0 < L; z0 += 32) {
                const int z = z0 + lane;
                double az = 0;
                for (int64_t b = 0; b < D2; ++b)
                    if (z < L && ((other[b] >> z) & 1)) az += ri[b] * rj[b];
                if (z < L) dz[p * L + z] = az;
            }
        }
    }
}

// Step 2: per-slot ordered sums of +/- densities.
__global__ void k_slot_gather(const uint32_t *__restrict__ ptr, const uint32_t *__restrict__ idx,
                              const int8_t *__restrict__ coef, const double *__restrict__ dens, int64_t nslots,
                              double *__restrict__ acc, int64_t ndens, unsigned long long *err) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nslots; s += (int64_t)gridDim.x * blockDim.x) {
        double v = 0;
        for (uint32_t e = ptr[s]; e < ptr[s + 1]; ++e) {
            const uint32_t k = idx[e];
            if (CIGPU_CHECK(err, index_ok(k, (uint64_t)ndens), kCheckRdmTerm, e)) v += (double)coef[e] * dens[k];
        }
        acc[s] = v;
    }
}

// Step 3: alpha-beta doubles. Block = (alpha excitation q = pidx(ar,ac), split);
// thread = beta excitation type (br, bc). slices[(q*nsplit + split)*L*L + br*L + bc].
__global__ void k_ab_doubles(const double *__restrict__ C, int64_t Db, const uint32_t *__restrict__ ap_ptr,
                             const uint64_t *__restrict__ ap, const int8_t *__restrict__ ap_sign,
                             const uint32_t *__restrict__ bx_ptr, const uint64_t *__restrict__ bx,
                             const int8_t *__restrict__ bx_sign, int L, int nsplit, double *__restrict__ slices,
                             int64_t Da, unsigned long long *err) {
    extern __shared__ double rows[];  // [2][Db]
    const int q = blockIdx.x / nsplit, split = blockIdx.x % nsplit;
    const uint32_t a0 = ap_ptr[q], a1 = ap_ptr[q + 1];
    const uint32_t cnt = a1 - a0, per = (cnt + nsplit - 1) / nsplit;
    const uint32_t s0 = a0 + min(cnt, split * per), s1 = a0 + min(cnt, (split + 1) * per);
    const int ntypes = L * L;
    constexpr int kMaxTypesPerThread = 8;
    double acc[kMaxTypesPerThread];
    for (int i = 0; i < kMaxTypesPerThread; ++i) acc[i] = 0;
    for (uint32_t e = s0; e < s1; ++e) {
        const uint64_t pr = ap[e];
        // the same pair for the whole block, so a skip keeps the barriers aligned
        if (!CIGPU_CHECK(err, index_ok((uint32_t)pr, (uint64_t)Da) && index_ok((uint32_t)(pr >> 32), (uint64_t)Da),
                         kCheckRdmPair, e))
            continue;
        const double *ri = C + (int64_t)(uint32_t)pr * Db;
        const double *rj = C + (int64_t)(uint32_t)(pr >> 32) * Db;
        __syncthreads();
        for (int64_t b = threadIdx.x; b < Db; b += blockDim.x) {
            rows[b] = ri[b];
            rows[Db + b] = rj[b];
        }
        __syncthreads();
        const double sa = (double)ap_sign[e];
        for (int i = 0; i < kMaxTypesPerThread; ++i) {
            const int ty = threadIdx.x + i * blockDim.x;
            if (ty >= ntypes) break;
            double part = 0;
            for (uint32_t x = bx_ptr[ty]; x < bx_ptr[ty + 1]; ++x) {
                const uint64_t bb = bx[x];
                if (!CIGPU_CHECK(err, index_ok((uint32_t)bb, (uint64_t)Db) && index_ok((uint32_t)(bb >> 32), (uint64_t)Db),
                                 kCheckRdmExcit, x))
                    continue;
                part += (double)bx_sign[x] * rows[(uint32_t)bb] * rows[Db + (uint32_t)(bb >> 32)];
            }
            acc[i] += sa * part;
        }
    }
    for (int i = 0; i < kMaxTypesPerThread; ++i) {
        const int ty = threadIdx.x + i * blockDim.x;
        if (ty < ntypes) slices[((int64_t)q * nsplit + split) * ntypes + ty] = acc[i];
    }
}

// Assemble the outputs: gather sums + alpha-beta double slices, mirrored.
__global__ void k_rdm_assemble(const double *__restrict__ acc, const double *__restrict__ slices, int nsplit, int L,
                               int np, size_t off_ga, size_t off_gb, size_t off_g0, size_t off_g1, size_t off_g2,
                               double *__restrict__ rdm1, double *__restrict__ aa, double *__restrict__ ab,
                               double *__restrict__ bb) {
    const int64_t L2 = (int64_t)L * L;
    const int64_t n1 = 2 * L2, n2 = (int64_t)np * np, n3 = L2 * L2;
    const int64_t total = n1 + 2 * n2 + n3;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < n1) {
            const int s = (int)(i / L2), a = (int)((i % L2) / L), b = (int)(i % L);
            rdm1[i] = acc[(s == 0 ? off_ga : off_gb) + (size_t)min(a, b) * L + max(a, b)];
        } else if (i < n1 + 2 * n2) {
            const int64_t j = i - n1;
            const int blk = (int)(j / n2);
            const int A = (int)((j % n2) / np), B = (int)(j % np);
            const double v = acc[(blk == 0 ? off_g0 : off_g2) + (size_t)min(A, B) * np + max(A, B)];
            (blk == 0 ? aa : bb)[j % n2] = v;
        } else {
            const int64_t j = i - n1 - 2 * n2;
            const int64_t A = j / L2, B = j % L2;
            const int64_t lo = min(A, B), hi = max(A, B);
            double v = acc[off_g1 + (size_t)lo * L2 + hi];
            const int ar = (int)(lo / L), ac = (int)(hi / L);
            if (ar < ac) {
                const int q = ar * L + ac - (ar + 1) * (ar + 2) / 2;
                const int64_t ty = (lo % L) * L + (hi % L);
                for (int sp = 0; sp < nsplit; ++sp) v += slices[((int64_t)q * nsplit + sp) * L2 + ty];
            }
            ab[j] = v;
        }
    }
}

__global__ void k_transpose(const double *__restrict__ a, int64_t rows, int64_t cols, double *__restrict__ t) {
    __shared__ double tile[32][33];
    const int64_t r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
        if (r0 + i < rows && c0 + threadIdx.x < cols) tile[i][threadIdx.x] = a[(r0 + i) * cols + c0 + threadIdx.x];
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
        if (c0 + i < cols && r0 + threadIdx.x < rows) t[(c0 + i) * rows + r0 + threadIdx.x] = tile[threadIdx.x][i];
}

// ---------------------------------------------------------------------------
// DOCI: thread (j,k) of an L*L block accumulates, over the block's pair strings,
//   A_jk = sum c_I^2 n_j n_k   and   B_jk = sum_{j in I, k not in I, k > j} c_I c_J,
// J = I - j + k. The block stages kDociChunk strings at a time in shared memory
// (one coalesced load of strings and c) with each string's rank prefix, so every
// pair-hop rank costs O(1): with p_1 < ... < p_n the occupied orbitals and
// rank(S) = sum_m C(p_m, m), moving the electron at j = p_{a+1} to the empty
// k > j (b electrons below k, j included) shifts p_{a+2..b} down one place:
//   rank(J) = I - C(j, a+1) + (P_b - P_{a+1}) + C(k, b),
//   P_m = sum_{i <= m} (C(p_i, i-1) - C(p_i, i)),
// evaluated modulo 2^32 (the result is a rank below 2^32, so the wrap cancels).
//
// The sums are 64-bit fixed-point integers (value * 2^60) on the integer pipe: a
// thread's FP64 add would occupy GB300's FP64 pipe (2 lanes per clock per SM) for
// the whole warp even when one lane of it needs the add, and most lanes of a warp
// skip a given string. Each coefficient becomes c * 2^62 (rounded to nearest, from
// its bit fields, |c| <= 1 for a normalised state), a product is the rounded high
// half of the 128-bit product (scale 2^60), and integer addition is associative, so
// the sums do not depend on order; each term is rounded by at most 2^-61 and every
// sum lies within +-1.
constexpr int kDociChunk = 128;
constexpr int kDociMaxL = 32;
constexpr int kRdmBatch = 8;  // pair hops gathered per round (loads in flight per thread)

// c * 2^62 rounded to nearest (|c| <= 1), from the IEEE-754 fields on the integer pipe.
__device__ __forceinline__ long long fx62(double c) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(c);
    const int e = (int)((u >> 52) & 0x7FF);
    if (e == 0) return 0;  // zero (and subnormals, below 2^-1022)
    const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int sh = e - 1013;  // c * 2^62 = m * 2^(e - 1023 - 52 + 62)
    unsigned long long r;
    if (sh >= 0)
        r = sh <= 10 ? (m << sh) : 0x4000000000000000ull;  // |c| <= 1 keeps sh <= 10
    else if (sh > -64)
        r = (m + (1ull << (-sh - 1))) >> (-sh);
    else
        r = 0;
    return (u >> 63) ? -(long long)r : (long long)r;
}

// (a * b) / 2^64 rounded to nearest: a, b at scale 2^62 give a product at 2^60.
__device__ __forceinline__ long long fxmul(long long a, long long b) {
    const long long hi = __mul64hi(a, b);
    const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
    return hi + (long long)(lo >> 63);
}

__global__ void k_doci_rdm(const double *__restrict__ c, const uint64_t *__restrict__ strings, int64_t D, int L,
                           int n, double *__restrict__ partial, unsigned long long *err) {
    __shared__ uint32_t binom[(kDociMaxL + 1) * (kDociMaxL + 2)];  // C(nn, kk), nn <= L, kk <= n + 1
    __shared__ uint64_t ss[kDociChunk];
    __shared__ long long cs[kDociChunk], cs2[kDociChunk];  // c_I * 2^62, c_I^2 * 2^60
    __shared__ uint32_t pre[kDociChunk][kDociMaxL + 1];
    constexpr int BW = kDociMaxL + 2;
    for (int i = threadIdx.x; i < (kDociMaxL + 1) * BW; i += blockDim.x) {
        const int nn = i / BW, kk = i % BW;
        binom[i] = (nn <= L && kk <= n + 1) ? (uint32_t)d_binom(nn, kk) : 0u;
    }
    // thread t owns the pair (j, k), j <= k, of the upper triangle in row-major
    // order (A is symmetric, B is summed for j < k only)
    const int t = threadIdx.x;
    const bool work = t < L * (L + 1) / 2;
    int j = 0, k = 0;
    if (work) {
        int rem = t;
        while (rem >= L - j) {
            rem -= L - j;
            ++j;
        }
        k = j + rem;
    }
    const bool hop = work && k > j;
    const uint64_t below_j = work ? (((uint64_t)1 << j) - 1) : 0, below_k = work ? (((uint64_t)1 << k) - 1) : 0;
    long long A = 0, B = 0;
    for (int64_t base = (int64_t)blockIdx.x * kDociChunk; base < D; base += (int64_t)gridDim.x * kDociChunk) {
        __syncthreads();  // the previous chunk is consumed (and the table is ready)
        const int cnt = (D - base) < kDociChunk ? (int)(D - base) : kDociChunk;
        for (int q = t; q < cnt; q += blockDim.x) {  // blocks of fewer than kDociChunk threads loop
            const uint64_t st = strings[base + q];
            const long long cf = fx62(c[base + q]);
            ss[q] = st;
            cs[q] = cf;
            cs2[q] = fxmul(cf, cf);
            uint32_t P = 0;
            pre[q][0] = 0;
            int m = 0;
            for (uint64_t x = st; x; x &= x - 1) {
                ++m;
                const int pm = __ffsll((long long)x) - 1;
                P += binom[pm * BW + m - 1] - binom[pm * BW + m];
                pre[q][m] = P;
            }
        }
        __syncthreads();
        if (work) {
            // kRdmBatch strings per round: ranks first, then their gathers of c
            // together, so several L2 loads are in flight per thread
            for (int i0 = 0; i0 < cnt; i0 += kRdmBatch) {
                uint32_t rr[kRdmBatch];
#pragma unroll
                for (int u = 0; u < kRdmBatch; ++u) {
                    const int i = i0 + u;
                    rr[u] = 0xFFFFFFFFu;
                    if (i < cnt) {
                        const uint64_t st = ss[i];
                        const bool nj = (st >> j) & 1, nk = (st >> k) & 1;
                        if (nj && nk) A += cs2[i];
                        if (hop && nj && !nk) {
                            const int a = __popcll(st & below_j), b = __popcll(st & below_k);
                            rr[u] = (uint32_t)(base + i) - binom[j * BW + a + 1] + pre[i][b] - pre[i][a + 1] +
                                    binom[k * BW + b];
                            if (!CIGPU_CHECK(err, index_ok(rr[u], (uint64_t)D), kCheckHopRank, rr[u])) rr[u] = 0xFFFFFFFFu;
                        }
                    }
                }
                double cv[kRdmBatch];
#pragma unroll
                for (int u = 0; u < kRdmBatch; ++u) cv[u] = rr[u] < (uint64_t)D ? __ldg(c + rr[u]) : 0.0;
#pragma unroll
                for (int u = 0; u < kRdmBatch; ++u)
                    if (rr[u] < (uint64_t)D) B += fxmul(cs[i0 + u], fx62(cv[u]));
            }
        }
    }
    // fixed-point sums at (j, k), j <= k, of the block's [2][L][L] partials (the
    // lower triangle is not written and not read), read back by the finishing kernels
    if (work) {
        long long *pl = reinterpret_cast<long long *>(partial);
        pl[((int64_t)blockIdx.x * 2) * L * L + j * L + k] = A;
        pl[((int64_t)blockIdx.x * 2 + 1) * L * L + j * L + k] = B;
    }
}

__global__ void k_doci_rdm_finish(const double *__restrict__ partial, int G, int L, int np, double *__restrict__ rdm1,
                                  double *__restrict__ aa, double *__restrict__ ab, double *__restrict__ bb) {
    const int L2 = L * L;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L2) return;
    const int j = t / L, k = t % L;
    const int tu = j <= k ? t : k * L + j;  // the partials hold j <= k
    const long long *pl = reinterpret_cast<const long long *>(partial);  // fixed point, 2^60
    long long Af = 0, Bf = 0;
    for (int b = 0; b < G; ++b) {
        Af += pl[((int64_t)b * 2) * L2 + tu];
        Bf += pl[((int64_t)b * 2 + 1) * L2 + tu];
    }
    const double A = (double)Af * 0x1p-60, B = (double)Bf * 0x1p-60;
    // 1-RDM (both spins): gamma_jj = A_jj
    if (j == k) {
        rdm1[j * L + j] = A;
        rdm1[L2 + j * L + j] = A;
    }
    // Gamma_ab(jk,jk) = A_jk; Gamma_ab(jj,kk) = Gamma_ab(kk,jj) = B_jk (j < k)
    ab[(int64_t)(j * L + k) * L2 + j * L + k] = A;
    if (j < k) {
        ab[(int64_t)(j * L + j) * L2 + k * L + k] = B;
        ab[(int64_t)(k * L + k) * L2 + j * L + j] = B;
        const int P = j * L + k - (j + 1) * (j + 2) / 2;
        aa[(int64_t)P * np + P] = A;
        bb[(int64_t)P * np + P] = A;
    }
}

// The two L x L matrices a DOCI state's RDMs reduce to, in CIDens element terms:
//   Pm[j][k] = get_two_rdm(1, j, j, k, k)   (pair hop B_jk; A_jj on the diagonal)
//   Dm[j][k] = get_two_rdm(0, j, k, j, k)   (A_jk; zero on the diagonal)
__global__ void k_doci_pairs_finish(const double *__restrict__ partial, int G, int L, double *__restrict__ Pm,
                                    double *__restrict__ Dm) {
    const int L2 = L * L;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L2) return;
    const int j = t / L, k = t % L;
    const int tu = j <= k ? t : k * L + j;  // the partials hold j <= k (B: j < k)
    const long long *pl = reinterpret_cast<const long long *>(partial);  // fixed point, 2^60
    long long Af = 0, Bf = 0;
    for (int b = 0; b < G; ++b) {
        Af += pl[((int64_t)b * 2) * L2 + tu];
        Bf += pl[((int64_t)b * 2 + 1) * L2 + tu];
    }
    const double A = (double)Af * 0x1p-60, B = (double)Bf * 0x1p-60;
    Pm[t] = j == k ? A : B;
    Dm[t] = j == k ? 0.0 : A;
}

template <typename T>
DevBuf<T> upload(const std::vector<T> &v, cudaStream_t s) {
    DevBuf<T> d(std::max<size_t>(v.size(), 1));
    if (!v.empty()) CIGPU_CUDA(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
}

}  // namespace

// The device copy of an FCI CRS's RDM plan: the string-pair lists, the per-element
// term lists and the alpha-beta excitation lists. It depends on the string tables
// only, so it is made on the first RDM call of a CRS and kept with it.
struct FciRdmPlan {
    int64_t npa = 0, nza = 0, npb = 0, nzb = 0;
    size_t ndens = 0, nslots = 0;
    size_t off_da0 = 0, off_daz = 0, off_db0 = 0, off_dbz = 0;
    size_t off_ga = 0, off_gb = 0, off_g0 = 0, off_g1 = 0, off_g2 = 0;
    int nsplit = 4;
    DevBuf<uint64_t> sa, sb;                  // alpha / beta strings
    DevBuf<uint32_t> aI, aJ, bI, bJ;          // string pairs per spin
    DevBuf<uint32_t> dptr, didx;              // terms of every RDM element (CSR)
    DevBuf<int8_t> dcf;
    DevBuf<uint32_t> app, bxp;                // alpha-beta doubles: alpha pairs per (ar<ac), beta per (br,bc)
    DevBuf<uint64_t> apd, bxd;
    DevBuf<int8_t> aps, bxs;
};

std::shared_ptr<FciRdmPlan> make_fci_rdm_plan(cigpu_crs &c, cudaStream_t s) {
    const int L = c.L, np = L * (L - 1) / 2;
    const int64_t L2 = (int64_t)L * L;
    const int64_t n2 = (int64_t)np * np, n3 = L2 * L2;
    const SpinTables &ta = c.ta;
    const SpinTables &tb = (c.ndown == c.nup) ? c.ta : c.tb;
    Plan P;
    P.L = L;
    P.np = np;
    P.Da = ta.D;
    P.Db = tb.D;
    P.off_ga = 0;
    P.off_gb = L2;
    P.off_g0 = 2 * L2;
    P.off_g2 = P.off_g0 + n2;
    P.off_g1 = P.off_g2 + n2;
    P.nslots = P.off_g1 + n3;
    // pair counts first (densities layout needs them)
    auto count_pairs = [&](const SpinTables &t, size_t &npair, size_t &nz) {
        size_t ns = 0, nd = 0;
        for (int64_t I = 0; I < t.D; ++I) {
            for (int q = 0; q < t.ns; ++q)
                if (t.s_target[(size_t)I * t.ns + q] > (uint32_t)I) ++ns;
            for (int q = 0; q < t.nd; ++q)
                if (t.d_target[(size_t)I * t.nd + q] > (uint32_t)I) ++nd;
        }
        nz = (size_t)t.D + ns;
        npair = nz + nd;
    };
    size_t npa, nza, npb, nzb;
    count_pairs(ta, npa, nza);
    count_pairs(tb, npb, nzb);
    P.off_da0 = 0;
    P.off_daz = npa;
    P.off_db0 = P.off_daz + nza * L;
    P.off_dbz = P.off_db0 + npb;
    P.ndens = P.off_dbz + nzb * L;
    plan_spin(P, ta, true);
    plan_spin(P, tb, false);
    plan_ab(P, ta, tb);
    if (P.a.I.size() != npa || P.b.I.size() != npb) throw std::runtime_error("rdm plan: pair count mismatch");
    // CSR of the slot terms: a stable counting sort keeps each slot's generation order
    std::vector<uint32_t> ptr(P.nslots + 1, 0), idx(P.terms.size());
    std::vector<int8_t> cf(P.terms.size());
    for (const auto &t : P.terms) ++ptr[t.slot + 1];
    for (size_t q = 0; q < P.nslots; ++q) ptr[q + 1] += ptr[q];
    {
        std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
        for (const auto &t : P.terms) {
            const uint32_t at = fill[t.slot]++;
            idx[at] = t.dens;
            cf[at] = t.coef;
        }
    }
    auto R = std::make_shared<FciRdmPlan>();
    R->npa = (int64_t)npa;
    R->nza = (int64_t)nza;
    R->npb = (int64_t)npb;
    R->nzb = (int64_t)nzb;
    R->ndens = P.ndens;
    R->nslots = P.nslots;
    R->off_da0 = P.off_da0;
    R->off_daz = P.off_daz;
    R->off_db0 = P.off_db0;
    R->off_dbz = P.off_dbz;
    R->off_ga = P.off_ga;
    R->off_gb = P.off_gb;
    R->off_g0 = P.off_g0;
    R->off_g1 = P.off_g1;
    R->off_g2 = P.off_g2;
    R->sa = upload(ta.strings, s);
    R->sb = upload(tb.strings, s);
    R->aI = upload(P.a.I, s);
    R->aJ = upload(P.a.J, s);
    R->bI = upload(P.b.I, s);
    R->bJ = upload(P.b.J, s);
    R->dptr = upload(ptr, s);
    R->didx = upload(idx, s);
    R->dcf = upload(cf, s);
    R->app = upload(P.ap_ptr, s);
    R->bxp = upload(P.bx_ptr, s);
    R->apd = upload(P.ap, s);
    R->bxd = upload(P.bx, s);
    R->aps = upload(P.ap_sign, s);
    R->bxs = upload(P.bx_sign, s);
    CIGPU_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
    return R;
}

void crs_rdm(cigpu_crs &c, const double *c_dev, double *rdm1, double *aa, double *ab, double *bb, cudaStream_t s) {
    if (c.method == CIGPU_DETS) {
        dets_rdm(c, c_dev, rdm1, aa, ab, bb, s);
        return;
    }
    const int L = c.L, np = L * (L - 1) / 2;
    const int64_t L2 = (int64_t)L * L;
    const int64_t n1 = 2 * L2, n2 = (int64_t)np * np, n3 = L2 * L2;
    DevBuf<double> out(n1 + 2 * n2 + n3);
    double *o1 = out.p, *oaa = out.p + n1, *obb = out.p + n1 + n2, *oab = out.p + n1 + 2 * n2;
    Trace tr("rdm", s);
    if (c.method == CIGPU_DOCI) {
        if (L * L > 1024) throw std::invalid_argument("DOCI RDM needs L <= 32");
        CIGPU_CUDA(cudaMemsetAsync(out.p, 0, sizeof(double) * out.n, s));
        const int G = sm_count() * 4;
        DevBuf<double> partial((size_t)G * 2 * L2);
        const int th = ((L * (L + 1) / 2 + 31) / 32) * 32;  // one thread per pair j <= k
        k_doci_rdm<<<G, th, 0, s>>>(c_dev, c.strings.p, c.dim, L, c.nup, partial.p, check_word_device());
        k_doci_rdm_finish<<<(int)((L2 + 255) / 256), 256, 0, s>>>(partial.p, G, L, np, o1, oaa, oab, obb);
        CIGPU_CUDA(cudaGetLastError());
        count_launch(2);
        CIGPU_CUDA(cudaStreamSynchronize(s));
        tr.mark("doci kernels");
    } else {
        if (L > 32) throw std::invalid_argument("FCI RDM needs L <= 32");
        if (!c.rdm_plan) {
            c.rdm_plan = make_fci_rdm_plan(c, s);
            tr.mark("host plan");
        }
        const FciRdmPlan &R = *c.rdm_plan;
        const SpinTables &ta = c.ta;
        const SpinTables &tb = (c.ndown == c.nup) ? c.ta : c.tb;
        // C^T for the beta densities
        DevBuf<double> Ct((size_t)c.dim);
        {
            dim3 grid((unsigned)((tb.D + 31) / 32), (unsigned)((ta.D + 31) / 32));
            k_transpose<<<grid, dim3(32, 8), 0, s>>>(c_dev, ta.D, tb.D, Ct.p);
            count_launch();
        }
        DevBuf<double> dens(R.ndens);
        const int G = sm_count() * 8;
        unsigned long long *ew = check_word_device();
        k_pair_dens<<<G, kRdmThreads, 0, s>>>(c_dev, tb.D, R.aI.p, R.aJ.p, R.npa, R.nza, R.sb.p, L,
                                              dens.p + R.off_da0, dens.p + R.off_daz, ta.D, ew);
        k_pair_dens<<<G, kRdmThreads, 0, s>>>(Ct.p, ta.D, R.bI.p, R.bJ.p, R.npb, R.nzb, R.sa.p, L,
                                              dens.p + R.off_db0, dens.p + R.off_dbz, tb.D, ew);
        count_launch(2);
        tr.mark("pair densities");
        DevBuf<double> acc(R.nslots);
        k_slot_gather<<<G, kRdmThreads, 0, s>>>(R.dptr.p, R.didx.p, R.dcf.p, dens.p, (int64_t)R.nslots, acc.p,
                                                (int64_t)R.ndens, ew);
        count_launch();
        tr.mark("slot sums");
        // alpha-beta doubles
        const int nsplit = R.nsplit;
        DevBuf<double> slices((size_t)std::max(np, 1) * nsplit * L2);
        if (np > 0) {
            const size_t sm = sizeof(double) * 2 * (size_t)tb.D;
            if (sm > 200 * 1024) throw std::invalid_argument("FCI RDM: beta string space too large");
            // one fixed limit, set once: concurrent callers (server workers) must never lower it
            static const cudaError_t attr =
                cudaFuncSetAttribute(k_ab_doubles, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            CIGPU_CUDA(attr);
            const int th = std::min(1024, (int)((L2 + 31) / 32 * 32));
            k_ab_doubles<<<np * nsplit, th, sm, s>>>(c_dev, tb.D, R.app.p, R.apd.p, R.aps.p, R.bxp.p, R.bxd.p,
                                                     R.bxs.p, L, nsplit, slices.p, ta.D, ew);
            count_launch();
        }
        tr.mark("alpha-beta doubles");
        k_rdm_assemble<<<G, kRdmThreads, 0, s>>>(acc.p, slices.p, nsplit, L, np, R.off_ga, R.off_gb, R.off_g0, R.off_g1,
                                                 R.off_g2, o1, oaa, oab, obb);
        CIGPU_CUDA(cudaGetLastError());
        count_launch();
        CIGPU_CUDA(cudaStreamSynchronize(s));
    }
    if (rdm1) CIGPU_CUDA(cudaMemcpyAsync(rdm1, o1, sizeof(double) * n1, cudaMemcpyDeviceToHost, s));
    if (aa) CIGPU_CUDA(cudaMemcpyAsync(aa, oaa, sizeof(double) * n2, cudaMemcpyDeviceToHost, s));
    if (bb) CIGPU_CUDA(cudaMemcpyAsync(bb, obb, sizeof(double) * n2, cudaMemcpyDeviceToHost, s));
    if (ab) CIGPU_CUDA(cudaMemcpyAsync(ab, oab, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
    tr.mark("assemble + copy out");
}

int doci_pair_partials() { return sm_count() * 4; }

void doci_pair_matrices(cigpu_crs &c, const double *c_dev, double *partial, double *Pm, double *Dm, cudaStream_t s) {
    if (c.method != CIGPU_DOCI || c.L > 32) throw std::invalid_argument("DOCI pair matrices need a DOCI CRS, L <= 32");
    const int L = c.L, G = doci_pair_partials();
    const int th = ((L * (L + 1) / 2 + 31) / 32) * 32;  // one thread per pair j <= k
    k_doci_rdm<<<G, th, 0, s>>>(c_dev, c.strings.p, c.dim, L, c.nup, partial, check_word_device());
    k_doci_pairs_finish<<<(L * L + 255) / 256, 256, 0, s>>>(partial, G, L, Pm, Dm);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(2);
}

}  // namespace cigpu

// ---------------------------------------------------------------------------
// DOCI RDMs without any device allocation (cigpu_rdm_doci_noalloc).
//
// Some callers cannot allocate device memory at the point where they need the
// RDMs: a host framework that hands out all device memory from its own fixed
// pool and forbids cudaMalloc on its request path, or a latency-bound loop where
// the implicit device synchronisation of cudaMalloc/cudaFree would stall work
// queued by others. For them the per-block partial sums of the DOCI RDM kernel
// live in a fixed array inside this library instead of in allocated scratch.
//
// The array below is file-scope device memory: every GPU that loads the library
// holds it (4 MiB) until the process exits. Host code must not take its name as
// a device address; the address is looked up once per device with
// cudaGetSymbolAddress (on the first call on that device, which should therefore
// come before any stream capture) and kept for the life of the process, so it
// does not survive a cudaDeviceReset of that device. The call runs on the current
// device, which must be the one the CRS was built on (CIGPU_EINVAL otherwise).
// Every call shares the array and leaves its contents behind: calls that overlap
// on the GPU race on it.
namespace cigpu {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;  // 4 MiB
constexpr int kNoAllocMaxBlocks = 256;

static __device__ __align__(256) double g_doci_rdm_scratch[kNoAllocScratchBytes / sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (set up once per device).
cudaError_t scratch_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_doci_rdm_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace cigpu

extern "C" int cigpu_rdm_doci_noalloc(cigpu_crs *crs, const double *c, double *rdm1, double *rdm2_aa,
                                      double *rdm2_ab, double *rdm2_bb, cigpu_stream stream) {
    using namespace cigpu;
    if (!crs || !c || !rdm1 || !rdm2_aa || !rdm2_ab || !rdm2_bb) return CIGPU_EINVAL;
    if (crs->method != CIGPU_DOCI) return CIGPU_EINVAL;
    const int L = crs->L, np = L * (L - 1) / 2;
    const int64_t L2 = (int64_t)L * L;
    // one thread per orbital pair (j, k) and 2 L^2 partial sums per block must fit
    if (L2 > 1024) return CIGPU_ENOTSUP;
    const int G = (int)std::min<int64_t>(kNoAllocMaxBlocks, kNoAllocScratchBytes / (sizeof(double) * 2 * L2));
    if (G < 1) return CIGPU_ENOTSUP;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return CIGPU_ECUDA;
    if (dev != crs->device) return CIGPU_EINVAL;  // the matrix and the scratch must share a device
    double *scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "cigpu: scratch address lookup failed: %s\n", cudaGetErrorString(e));
        return CIGPU_ECUDA;
    }
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : crs->stream;
    // the finishing kernel only writes the nonzero DOCI entries: clear the outputs
    if (cudaMemsetAsync(rdm1, 0, sizeof(double) * 2 * L2, s) != cudaSuccess ||
        cudaMemsetAsync(rdm2_aa, 0, sizeof(double) * np * np, s) != cudaSuccess ||
        cudaMemsetAsync(rdm2_bb, 0, sizeof(double) * np * np, s) != cudaSuccess ||
        cudaMemsetAsync(rdm2_ab, 0, sizeof(double) * L2 * L2, s) != cudaSuccess)
        return CIGPU_ECUDA;
    const int th = (int)((L2 + 31) / 32 * 32);
    k_doci_rdm<<<G, th, 0, s>>>(c, crs->strings.p, crs->dim, L, crs->nup, scratch, nullptr);  // no error word: allocates nothing
    k_doci_rdm_finish<<<(int)((L2 + 255) / 256), 256, 0, s>>>(scratch, G, L, np, rdm1, rdm2_aa, rdm2_ab, rdm2_bb);
    if (cudaGetLastError() != cudaSuccess) return CIGPU_ECUDA;
    count_launch(2);
    return CIGPU_OK;
}
