/* CPU restatement of the CIFlow lowest-eigenpair CI path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path; only tests/, the
 * smoke check and bench.py's CPU-baseline leg load it.
 *
 * Each routine restates the reference algorithm it cites (paths relative to
 * the CIFlow tree). The build keeps the reference's loop order, its sorted
 * row insertion with add / overwrite semantics and its 1e-14 drop threshold,
 * so the CRS it emits is the reference CRS; the element functions keep the
 * reference's order of floating-point additions, so values agree bit for bit.
 */
#include "ciflow_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint64_t bits_t;

/* SparseMatrix_CRS::_zero (SparseMatrix_CRS.cpp:44). */
#define ORC_ZERO 1e-14

typedef struct {
    int L, na, nb;
    const double *h;
    const double *eri;
    size_t L1, L2, L3;
} ham_t;

static inline double T(const ham_t *H, int i, int j) { return H->h[(size_t)i * H->L1 + j]; }
/* Physics <ij|kl> = chemist (ik|jl) (Hamiltonian.h:45, Hamiltonian.cpp:873). */
static inline double V(const ham_t *H, int i, int j, int k, int l) {
    return H->eri[(size_t)i * H->L3 + (size_t)k * H->L2 + (size_t)j * H->L1 + l];
}

int64_t orc_binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

int64_t orc_dim(int method, int L, int nup, int ndown) {
    if (method == ORC_DOCI) return orc_binom(L, nup);
    return orc_binom(L, nup) * orc_binom(L, ndown);
}

/* Permutator_Bit::get_start_int / permutate_bit (Permutator.cpp:146-153, 113-119):
 * Gosper's next combination, i.e. colex order. */
static inline bits_t first_string(int n) { return n >= 64 ? ~(bits_t)0 : (((bits_t)1 << n) - 1); }
static inline bits_t next_string(bits_t v) {
    bits_t t = v | (v - 1);
    return (t + 1) | (((~t & -~t) - 1) >> (__builtin_ctzll(v) + 1));
}

/* determine_weight (CIMethod.cpp:689-704): rank = sum_m C(p_m, m), m = 1..n over set bits. */
static inline uint32_t string_rank(bits_t s, const int64_t *binom_tab, int L) {
    int64_t w = 0;
    int m = 0;
    for (int k = 0; k < L; ++k)
        if (s & ((bits_t)1 << k)) {
            ++m;
            w += binom_tab[k * 65 + m];
        }
    return (uint32_t)w;
}

static int64_t *make_binom_tab(void) {
    int64_t *t = (int64_t *)calloc(65 * 65, sizeof(int64_t));
    for (int n = 0; n <= 64; ++n)
        for (int k = 0; k <= 64; ++k) t[n * 65 + k] = (n <= 62) ? orc_binom(n, k) : 0;
    return t;
}

/* get_orbs (CIMethod.cpp:313-327): ascending occupied orbitals. */
static inline int get_orbs(bits_t s, int *o) {
    int n = 0;
    while (s) {
        o[n++] = __builtin_ctzll(s);
        s &= s - 1;
    }
    return n;
}

/* get_nstacked (CIMethod.cpp:382-396): set bits of `up` in [min(o0,o1), max(o0,o1)). */
static inline int nstacked(int o0, int o1, bits_t up) {
    int lo = o0 < o1 ? o0 : o1, hi = o0 < o1 ? o1 : o0;
    int sum = 0;
    for (int i = lo; i < hi; ++i)
        if (up & ((bits_t)1 << i)) ++sum;
    return sum;
}

/* arrange_order (CIMethod.cpp:353-380): orbitals of up1 first, then those of up2,
 * ascending within each group. */
static inline void arrange_order(int *orbs, int num, bits_t up1) {
    int re[4];
    int a = 0, b = (num == 4) ? 2 : 1;
    for (int i = 0; i < num; ++i) {
        if (up1 & ((bits_t)1 << orbs[i]))
            re[a++] = orbs[i];
        else
            re[b++] = orbs[i];
    }
    for (int i = 0; i < num; ++i) orbs[i] = re[i];
}

/* get_diag_cont_one_bitstring (CIMethod.cpp:329-342). */
static double diag_one(const ham_t *H, const int *o, int n) {
    double s = 0;
    for (int k = 0; k < n; ++k) s += T(H, o[k], o[k]);
    for (int k = 0; k < n - 1; ++k)
        for (int l = k + 1; l < n; ++l) s += V(H, o[k], o[l], o[k], o[l]) - V(H, o[k], o[l], o[l], o[k]);
    return s;
}

/* CIMethod::diagonal (CIMethod.cpp:398-407) with get_diag_cont_jmix (:344-351). */
static double diagonal(const ham_t *H, bits_t up, bits_t dn) {
    int ou[64] = {0}, od[64] = {0};
    int nu = get_orbs(up, ou), nd = get_orbs(dn, od);
    double tot = diag_one(H, ou, nu);
    tot += diag_one(H, od, nd);
    double mix = 0;
    for (int k = 0; k < nu; ++k)
        for (int l = 0; l < nd; ++l) mix += V(H, ou[k], od[l], ou[k], od[l]);
    tot += mix;
    return tot;
}

/* one_diff_orbital (CIMethod.cpp:409-427); `other` is the opposite-spin string. */
static double one_diff(const ham_t *H, bits_t s1, bits_t s2, bits_t other) {
    int orbs[64], com[64], oth[64];
    get_orbs(s1 ^ s2, orbs);
    double e = T(H, orbs[0], orbs[1]);
    int nc = get_orbs(s1 & s2, com);
    for (int z = 0; z < nc; ++z)
        e += V(H, orbs[0], com[z], orbs[1], com[z]) - V(H, orbs[0], com[z], com[z], orbs[1]);
    int diff = nstacked(orbs[0], orbs[1], s1 & s2);
    int no = get_orbs(other, oth);
    for (int z = 0; z < no; ++z) e += V(H, orbs[0], oth[z], orbs[1], oth[z]);
    if (diff % 2 != 0) e *= -1;
    return e;
}

/* two_diff_orbitals(up1,up2) (CIMethod.cpp:429-442): same-spin double. */
static double two_diff_same(const ham_t *H, bits_t s1, bits_t s2) {
    int o[64];
    get_orbs(s1 ^ s2, o);
    arrange_order(o, 4, s1);
    bits_t c = s1 & s2;
    int diff = nstacked(o[0], o[1], c) + nstacked(o[2], o[3], c);
    double e = V(H, o[0], o[1], o[2], o[3]) - V(H, o[0], o[1], o[3], o[2]);
    if (diff % 2 != 0) e *= -1;
    return e;
}

/* two_diff_orbitals(up1,up2,down1,down2) (CIMethod.cpp:444-457): alpha-beta double. */
static double two_diff_ab(const ham_t *H, bits_t u1, bits_t u2, bits_t d1, bits_t d2) {
    int a[64], b[64];
    get_orbs(u1 ^ u2, a);
    get_orbs(d1 ^ d2, b);
    arrange_order(a, 2, u1);
    arrange_order(b, 2, d1);
    int diff = nstacked(a[0], a[1], u1 & u2) + nstacked(b[0], b[1], d1 & d2);
    double e = V(H, a[0], b[0], a[1], b[1]);
    if (diff % 2 != 0) e *= -1;
    return e;
}

/* ---- one CRS row under construction: NewRow/PushToRow/PushToRownoadd
 *      (SparseMatrix_CRS.cpp:240-322) ---- */
typedef struct {
    uint32_t *col;
    double *val;
    int n;
} rowbuf_t;

static void push_row(rowbuf_t *r, uint32_t j, double v, int add) {
    if (!(fabs(v) > ORC_ZERO)) return;
    if (r->n == 0 || r->col[r->n - 1] < j) {
        r->col[r->n] = j;
        r->val[r->n] = v;
        r->n++;
        return;
    }
    for (int i = 0; i < r->n; ++i) {
        if (r->col[i] > j) {
            memmove(r->col + i + 1, r->col + i, (size_t)(r->n - i) * sizeof(uint32_t));
            memmove(r->val + i + 1, r->val + i, (size_t)(r->n - i) * sizeof(double));
            r->col[i] = j;
            r->val[i] = v;
            r->n++;
            return;
        }
        if (r->col[i] == j) {
            if (add) {
                r->val[i] += v;
                if (fabs(r->val[i]) < ORC_ZERO) {
                    memmove(r->col + i, r->col + i + 1, (size_t)(r->n - i - 1) * sizeof(uint32_t));
                    memmove(r->val + i, r->val + i + 1, (size_t)(r->n - i - 1) * sizeof(double));
                    r->n--;
                }
            } else {
                r->val[i] = v;
            }
            return;
        }
    }
}

/* FCI::construct_CI_matrix for one row (CIMethod.cpp:766-883). */
static void fci_row(const ham_t *H, const int64_t *bt, bits_t up1, bits_t down1, long i, long k, long Dd,
                    rowbuf_t *r) {
    const int L = H->L;
    r->n = 0;
    push_row(r, (uint32_t)(i * Dd + k), diagonal(H, up1, down1), 1);
    for (int j = 0; j < L; ++j) {
        if (!(up1 & ((bits_t)1 << j))) continue;
        bits_t up_interm = up1 ^ ((bits_t)1 << j);
        for (int l = j + 1; l < L; ++l) {
            if (up1 & ((bits_t)1 << l)) continue;
            bits_t up2 = up_interm ^ ((bits_t)1 << l);
            uint32_t index = string_rank(up2, bt, L);
            push_row(r, (uint32_t)(index * Dd + k), one_diff(H, up1, up2, down1), 1);
            for (int m = 0; m < L; ++m) {
                if (!(down1 & ((bits_t)1 << m))) continue;
                bits_t down_interm = down1 ^ ((bits_t)1 << m);
                for (int w = 0; w < L; ++w) {
                    if (down1 & ((bits_t)1 << w)) continue;
                    bits_t down2 = down_interm ^ ((bits_t)1 << w);
                    uint32_t indexd = string_rank(down2, bt, L);
                    push_row(r, (uint32_t)(index * Dd + indexd), two_diff_ab(H, up1, up2, down1, down2), 1);
                }
            }
            for (int m = 0; m < L; ++m) {
                if (!((up2 & ((bits_t)1 << m)) && m != l)) continue;
                bits_t ups_interm = up2 ^ ((bits_t)1 << m);
                for (int w = 0; w < L; ++w) {
                    if ((up2 & ((bits_t)1 << w)) || w == j) continue;
                    bits_t updex = ups_interm ^ ((bits_t)1 << w);
                    uint32_t indexdex = string_rank(updex, bt, L);
                    if ((long)indexdex > i) push_row(r, (uint32_t)(indexdex * Dd + k), two_diff_same(H, up1, updex), 0);
                }
            }
        }
    }
    for (int j = 0; j < L; ++j) {
        if (!(down1 & ((bits_t)1 << j))) continue;
        bits_t down_interm = down1 ^ ((bits_t)1 << j);
        for (int l = j + 1; l < L; ++l) {
            if (down1 & ((bits_t)1 << l)) continue;
            bits_t down2 = down_interm ^ ((bits_t)1 << l);
            uint32_t index = string_rank(down2, bt, L);
            push_row(r, (uint32_t)(i * Dd + index), one_diff(H, down1, down2, up1), 1);
            for (int m = 0; m < L; ++m) {
                if (!((down2 & ((bits_t)1 << m)) && m != l)) continue;
                bits_t downs_interm = down2 ^ ((bits_t)1 << m);
                for (int w = 0; w < L; ++w) {
                    if ((down2 & ((bits_t)1 << w)) || w == j) continue;
                    bits_t downdex = downs_interm ^ ((bits_t)1 << w);
                    uint32_t indexddex = string_rank(downdex, bt, L);
                    if ((long)indexddex > k)
                        push_row(r, (uint32_t)(i * Dd + indexddex), two_diff_same(H, down1, downdex), 0);
                }
            }
        }
    }
}

/* DOCI::construct_CI_matrix for one row (CIMethod.cpp:623-656). */
static void doci_row(const ham_t *H, const int64_t *bt, bits_t up1, long i, rowbuf_t *r) {
    const int L = H->L;
    r->n = 0;
    (void)i;
    push_row(r, (uint32_t)i, diagonal(H, up1, up1), 1);
    for (int j = 0; j < L; ++j) {
        if (!(up1 & ((bits_t)1 << j))) continue;
        bits_t up_interm = up1 ^ ((bits_t)1 << j);
        for (int k = j + 1; k < L; ++k) {
            if (up1 & ((bits_t)1 << k)) continue;
            bits_t up2 = up_interm ^ ((bits_t)1 << k);
            uint32_t index = string_rank(up2, bt, L);
            push_row(r, index, two_diff_ab(H, up1, up2, up1, up2), 1);
        }
    }
}

static bits_t *enumerate_strings(int L, int n, int64_t D) {
    bits_t *s = (bits_t *)malloc((size_t)D * sizeof(bits_t));
    bits_t v = first_string(n);
    for (int64_t i = 0; i < D; ++i) {
        s[i] = v;
        v = next_string(v);
    }
    (void)L;
    return s;
}

int orc_build_upper(int method, int L, int nup, int ndown, const double *h, const double *eri, int64_t *row,
                    uint32_t *col, double *val) {
    if (L < 1 || L > 62 || nup < 0 || ndown < 0 || nup > L || ndown > L) return 1;
    if (method == ORC_DOCI && nup != ndown) return 1;
    ham_t H = {L, nup, ndown, h, eri, (size_t)L, (size_t)L * L, (size_t)L * L * L};
    int64_t *bt = make_binom_tab();
    const int64_t Du = orc_binom(L, nup), Dd = (method == ORC_DOCI) ? 1 : orc_binom(L, ndown);
    const int64_t dim = Du * Dd;
    bits_t *us = enumerate_strings(L, nup, Du);
    bits_t *ds = (method == ORC_DOCI) ? NULL : enumerate_strings(L, ndown, Dd);
    const int64_t sa = (int64_t)nup * (L - nup), sb = (int64_t)ndown * (L - ndown);
    const int64_t wmax = 2 + sa + sb + sa * sb + orc_binom(nup, 2) * orc_binom(L - nup, 2) +
                         orc_binom(ndown, 2) * orc_binom(L - ndown, 2);
    const int fill = (col != NULL);
    int64_t *counts = NULL;
    if (!fill) counts = row + 1;

#pragma omp parallel
    {
        rowbuf_t r;
        r.col = (uint32_t *)malloc((size_t)wmax * sizeof(uint32_t));
        r.val = (double *)malloc((size_t)wmax * sizeof(double));
        if (method == ORC_DOCI) {
#pragma omp for schedule(dynamic, 256)
            for (int64_t i = 0; i < Du; ++i) {
                doci_row(&H, bt, us[i], (long)i, &r);
                if (!fill) {
                    counts[i] = r.n;
                } else {
                    memcpy(col + row[i], r.col, (size_t)r.n * sizeof(uint32_t));
                    memcpy(val + row[i], r.val, (size_t)r.n * sizeof(double));
                }
            }
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int64_t i = 0; i < Du; ++i) {
                for (int64_t k = 0; k < Dd; ++k) {
                    const int64_t rr = i * Dd + k;
                    fci_row(&H, bt, us[i], ds[k], (long)i, (long)k, (long)Dd, &r);
                    if (!fill) {
                        counts[rr] = r.n;
                    } else {
                        memcpy(col + row[rr], r.col, (size_t)r.n * sizeof(uint32_t));
                        memcpy(val + row[rr], r.val, (size_t)r.n * sizeof(double));
                    }
                }
            }
        }
        free(r.col);
        free(r.val);
    }
    if (!fill) {
        row[0] = 0;
        for (int64_t i = 0; i < dim; ++i) row[i + 1] += row[i];
    }
    free(us);
    free(ds);
    free(bt);
    return 0;
}

/* SparseMatrix_CRS_Sym::mvprod (SparseMatrix_CRS.cpp:700-723), serial. */
void orc_sym_mvprod(int64_t n, const int64_t *row, const uint32_t *col, const double *val, const double *x,
                    double *y) {
    for (int64_t i = 0; i < n; ++i) y[i] = 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t k = row[i]; k < row[i + 1]; ++k) {
            y[i] += val[k] * x[col[k]];
            if ((uint32_t)i != col[k]) y[col[k]] += val[k] * x[i];
        }
    }
}

void orc_sym_mvprod_omp(int64_t n, const int64_t *row, const uint32_t *col, const double *val, const double *x,
                        double *y) {
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    double *buf = (double *)calloc((size_t)nt * (size_t)n, sizeof(double));
#pragma omp parallel
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double *yt = buf + (size_t)t * n;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n; ++i) {
            double acc = 0;
            const double xi = x[i];
            for (int64_t k = row[i]; k < row[i + 1]; ++k) {
                acc += val[k] * x[col[k]];
                if ((uint32_t)i != col[k]) yt[col[k]] += val[k] * xi;
            }
            yt[i] += acc;
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double s = 0;
            for (int q = 0; q < nt; ++q) s += buf[(size_t)q * n + i];
            y[i] = s;
        }
    }
    free(buf);
}

/* ---------------- RDMs (CIDens.cpp) ---------------- */

typedef struct {
    int L, np;
    double *one;  /* [2][L][L], accumulated at (min,max) */
    double *aa;   /* [np][np], accumulated at (min,max) */
    double *ab;   /* [L*L][L*L] */
    double *bb;
} rdm_t;

static size_t rdm_size(int L) {
    size_t np = (size_t)L * (L - 1) / 2;
    return 2 * (size_t)L * L + 2 * np * np + (size_t)L * L * L * L;
}

static void rdm_bind(rdm_t *R, int L, double *base) {
    R->L = L;
    R->np = L * (L - 1) / 2;
    R->one = base;
    R->aa = R->one + 2 * (size_t)L * L;
    R->bb = R->aa + (size_t)R->np * R->np;
    R->ab = R->bb + (size_t)R->np * R->np;
}

/* add_one_rdm (CIDens.cpp:280-292): upper-packed symmetric storage. */
static inline void add_one(rdm_t *R, int spin, int o1, int o2, double v) {
    int a = o1 < o2 ? o1 : o2, b = o1 < o2 ? o2 : o1;
    R->one[((size_t)spin * R->L + a) * R->L + b] += v;
}

static inline int pidx(int p, int q, int L) { return p * L + q - (p + 1) * (p + 2) / 2; }

/* add_two_rdm (CIDens.cpp:227-256) into the symmetric pair-matrix Vector2d
 * storage (matrix.cpp:674-690). */
static inline void add_two(rdm_t *R, int spin, int o1, int o2, int o3, int o4, double v) {
    const int L = R->L;
    if (spin == 1) {
        size_t A = (size_t)o1 * L + o2, B = (size_t)o3 * L + o4;
        size_t a = A < B ? A : B, b = A < B ? B : A;
        R->ab[a * (size_t)L * L + b] += v;
        return;
    }
    if (o1 == o2 || o3 == o4) return;
    if (o1 > o2) {
        int t = o1; o1 = o2; o2 = t; v = -v;
    }
    if (o3 > o4) {
        int t = o3; o3 = o4; o4 = t; v = -v;
    }
    size_t A = pidx(o1, o2, L), B = pidx(o3, o4, L);
    size_t a = A < B ? A : B, b = A < B ? B : A;
    double *X = (spin == 0) ? R->aa : R->bb;
    X[a * R->np + b] += v;
}

/* fill_one_dense (CIDens.cpp:676-754). mode 0/1: 1-RDM alpha/beta; 2: 2-RDM from an
 * alpha single; 3: 2-RDM from a beta single. */
static void fill_one_dense(rdm_t *R, bits_t b1, bits_t b2, bits_t same, double contr, int mode) {
    int orbs[64], other[64], so[64];
    get_orbs(b1 ^ b2, orbs);
    int no = get_orbs(b1 & b2, other);
    int ns = get_orbs(same, so);
    if (nstacked(orbs[0], orbs[1], b1 & b2) % 2 != 0) contr *= -1;
    if (mode < 2) {
        add_one(R, mode, orbs[0], orbs[1], contr);
    } else if (mode == 2) {
        for (int i = 0; i < no; ++i) add_two(R, 0, orbs[0], other[i], orbs[1], other[i], contr);
        for (int i = 0; i < ns; ++i) add_two(R, 1, orbs[0], so[i], orbs[1], so[i], contr);
    } else {
        for (int i = 0; i < no; ++i) add_two(R, 2, orbs[0], other[i], orbs[1], other[i], contr);
        for (int i = 0; i < ns; ++i) add_two(R, 1, so[i], orbs[0], so[i], orbs[1], contr);
    }
}

/* fill_two_dense (CIDens.cpp:756-779). */
static void fill_two_dense(rdm_t *R, bits_t s1, bits_t s2, double contr, int spin) {
    int o[64];
    get_orbs(s1 ^ s2, o);
    arrange_order(o, 4, s1);
    int diff = nstacked(o[0], o[1], s1 & s2) + nstacked(o[2], o[3], s1 & s2);
    if (diff % 2 != 0) contr *= -1;
    add_two(R, spin, o[0], o[1], o[2], o[3], contr);
}

/* fill_two_dense_upanddown (CIDens.cpp:781-806). */
static void fill_two_ud(rdm_t *R, bits_t u1, bits_t u2, bits_t d1, bits_t d2, double contr) {
    int a[64], b[64];
    get_orbs(u1 ^ u2, a);
    get_orbs(d1 ^ d2, b);
    arrange_order(a, 2, u1);
    arrange_order(b, 2, d1);
    int diff = nstacked(a[0], a[1], u1 & u2) + nstacked(b[0], b[1], d1 & d2);
    if (diff % 2 != 0) contr *= -1;
    add_two(R, 1, a[0], b[0], a[1], b[1], contr);
}

/* fill_diagonal (CIDens.cpp:808-853). */
static void fill_diagonal(rdm_t *R, bits_t up, bits_t dn, double contr, int two) {
    int ou[64], od[64];
    int nu = get_orbs(up, ou), nd = get_orbs(dn, od);
    for (int i = 0; i < nu; ++i) {
        if (!two)
            add_one(R, 0, ou[i], ou[i], contr);
        else
            for (int j = i + 1; j < nu; ++j) add_two(R, 0, ou[i], ou[j], ou[i], ou[j], contr);
    }
    for (int i = 0; i < nd; ++i) {
        if (!two)
            add_one(R, 1, od[i], od[i], contr);
        else
            for (int j = i + 1; j < nd; ++j) add_two(R, 2, od[i], od[j], od[i], od[j], contr);
    }
    if (two)
        for (int i = 0; i < nu; ++i)
            for (int j = 0; j < nd; ++j) add_two(R, 1, ou[i], od[j], ou[i], od[j], contr);
}

/* fill_density_matrix (CIDens.cpp:855-881). */
static void fill_pair_two(rdm_t *R, bits_t u1, bits_t d1, bits_t u2, bits_t d2, double contr) {
    int pu = __builtin_popcountll(u1 ^ u2), pd = __builtin_popcountll(d1 ^ d2);
    if (pd > 4 || pu > 4) return;
    if (pu == 4 && pd == 0)
        fill_two_dense(R, u1, u2, contr, 0);
    else if (pu == 2) {
        if (pd == 0)
            fill_one_dense(R, u1, u2, d1, contr, 2);
        else if (pd == 2)
            fill_two_ud(R, u1, u2, d1, d2, contr);
    } else if (pd == 4 && pu == 0)
        fill_two_dense(R, d1, d2, contr, 2);
    else if (pd == 2 && pu == 0)
        fill_one_dense(R, d1, d2, u1, contr, 3);
    else if (pd == 0 && pu == 0)
        fill_diagonal(R, u1, d1, contr, 1);
}

/* fill_density_matrix_one (CIDens.cpp:883-896). */
static void fill_pair_one(rdm_t *R, bits_t u1, bits_t d1, bits_t u2, bits_t d2, double contr) {
    int pu = __builtin_popcountll(u1 ^ u2), pd = __builtin_popcountll(d1 ^ d2);
    if (pu > 2 || pd > 2) return;
    if (pu == 2 && pd == 0)
        fill_one_dense(R, u1, u2, d1, contr, 0);
    else if (pu == 0 && pd == 2)
        fill_one_dense(R, d1, d2, u1, contr, 1);
    else if (pu == 0 && pd == 0)
        fill_diagonal(R, u1, d1, contr, 0);
}

/* Expand the (min,max)-accumulated storage into full symmetric matrices. */
static void rdm_finish(const rdm_t *R, double *rdm1, double *aa, double *ab, double *bb) {
    const int L = R->L, np = R->np;
    const size_t L2 = (size_t)L * L;
    for (int s = 0; s < 2; ++s)
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                int a = i < j ? i : j, b = i < j ? j : i;
                rdm1[((size_t)s * L + i) * L + j] = R->one[((size_t)s * L + a) * L + b];
            }
    for (int i = 0; i < np; ++i)
        for (int j = 0; j < np; ++j) {
            int a = i < j ? i : j, b = i < j ? j : i;
            aa[(size_t)i * np + j] = R->aa[(size_t)a * np + b];
            bb[(size_t)i * np + j] = R->bb[(size_t)a * np + b];
        }
    for (size_t i = 0; i < L2; ++i)
        for (size_t j = 0; j < L2; ++j) {
            size_t a = i < j ? i : j, b = i < j ? j : i;
            ab[i * L2 + j] = R->ab[a * L2 + b];
        }
}

/* Per-thread accumulation buffers, summed in thread order. */
typedef struct {
    int nt;
    size_t sz;
    double *buf;
} rdm_pool_t;

static void pool_init(rdm_pool_t *P, int L) {
    P->nt = 1;
#ifdef _OPENMP
    P->nt = omp_get_max_threads();
#endif
    P->sz = rdm_size(L);
    P->buf = (double *)calloc((size_t)P->nt * P->sz, sizeof(double));
}

static void pool_reduce(rdm_pool_t *P, int L, double *rdm1, double *aa, double *ab, double *bb) {
    for (int t = 1; t < P->nt; ++t)
        for (size_t i = 0; i < P->sz; ++i) P->buf[i] += P->buf[(size_t)t * P->sz + i];
    rdm_t R;
    rdm_bind(&R, L, P->buf);
    rdm_finish(&R, rdm1, aa, ab, bb);
    free(P->buf);
}

static int thread_id(void) {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

/* DensDOCI::construct_CI_one_dens / construct_CI_two_dens (CIDens.cpp:1073-1224). */
static void doci_rdm(int L, int np_, const double *c, rdm_pool_t *P) {
    const int64_t D = orc_binom(L, np_);
    bits_t *us = enumerate_strings(L, np_, D);
    int64_t *bt = make_binom_tab();
#pragma omp parallel
    {
        rdm_t R;
        rdm_bind(&R, L, P->buf + (size_t)thread_id() * P->sz);
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < D; ++i) {
            const bits_t up1 = us[i];
            const double contr = c[i] * c[i];
            for (int j = 0; j < L; ++j)
                if (up1 & ((bits_t)1 << j)) {
                    add_one(&R, 0, j, j, contr);
                    add_one(&R, 1, j, j, contr);
                }
            for (int j = 0; j < L; ++j) {
                if (!(up1 & ((bits_t)1 << j))) continue;
                for (int k = j; k < L; ++k) {
                    if (!(up1 & ((bits_t)1 << k))) continue;
                    if (j != k) {
                        add_two(&R, 0, j, k, j, k, contr);
                        add_two(&R, 2, j, k, j, k, contr);
                        add_two(&R, 1, k, j, k, j, contr);
                    }
                    add_two(&R, 1, j, k, j, k, contr);
                }
                bits_t up_interm = up1 ^ ((bits_t)1 << j);
                for (int k = j + 1; k < L; ++k) {
                    if (up1 & ((bits_t)1 << k)) continue;
                    bits_t up2 = up_interm ^ ((bits_t)1 << k);
                    uint32_t index = string_rank(up2, bt, L);
                    add_two(&R, 1, j, j, k, k, c[i] * c[index]);
                }
            }
        }
    }
    free(us);
    free(bt);
}

int orc_rdm_pairs(int method, int L, int nup, int ndown, const double *c, double *rdm1, double *aa, double *ab,
                  double *bb) {
    if (L < 2 || L > 62) return 1;
    rdm_pool_t P;
    pool_init(&P, L);
    if (method == ORC_DOCI) {
        doci_rdm(L, nup, c, &P);
    } else {
        const int64_t Du = orc_binom(L, nup), Dd = orc_binom(L, ndown);
        bits_t *us = enumerate_strings(L, nup, Du);
        bits_t *ds = enumerate_strings(L, ndown, Dd);
#pragma omp parallel
        {
            rdm_t R;
            rdm_bind(&R, L, P.buf + (size_t)thread_id() * P.sz);
            /* DensFCI::construct_CI_one_dens (CIDens.cpp:1530-1580). */
#pragma omp for schedule(dynamic, 1)
            for (int64_t i = 0; i < Du; ++i) {
                for (int64_t j = i; j < Du; ++j)
                    for (int64_t k = 0; k < Dd; ++k)
                        fill_pair_one(&R, us[i], ds[k], us[j], ds[k], c[i * Dd + k] * c[j * Dd + k]);
                for (int64_t k = 0; k < Dd - 1; ++k)
                    for (int64_t j = k + 1; j < Dd; ++j)
                        fill_pair_one(&R, us[i], ds[k], us[i], ds[j], c[i * Dd + k] * c[i * Dd + j]);
            }
            /* DensFCI::construct_CI_two_dens (CIDens.cpp:1582-1631). */
#pragma omp for schedule(dynamic, 1)
            for (int64_t i = 0; i < Du; ++i) {
                for (int64_t j = i + 1; j < Du; ++j)
                    for (int64_t k = 0; k < Dd; ++k)
                        for (int64_t l = 0; l < Dd; ++l)
                            fill_pair_two(&R, us[i], ds[k], us[j], ds[l], c[i * Dd + k] * c[j * Dd + l]);
                for (int64_t k = 0; k < Dd; ++k)
                    for (int64_t l = k; l < Dd; ++l)
                        fill_pair_two(&R, us[i], ds[k], us[i], ds[l], c[i * Dd + k] * c[i * Dd + l]);
            }
        }
        free(us);
        free(ds);
    }
    pool_reduce(&P, L, rdm1, aa, ab, bb);
    return 0;
}

/* The same contributions as orc_rdm_pairs for FCI, but each row I only visits
 * the determinants J > I it is connected to (diagonal, singles, doubles), so the
 * cost is O(dim * connections) instead of O(dim^2). */
int orc_rdm_excitations(int method, int L, int nup, int ndown, const double *c, double *rdm1, double *aa,
                        double *ab, double *bb) {
    if (method == ORC_DOCI) return orc_rdm_pairs(method, L, nup, ndown, c, rdm1, aa, ab, bb);
    if (L < 2 || L > 62) return 1;
    rdm_pool_t P;
    pool_init(&P, L);
    const int64_t Du = orc_binom(L, nup), Dd = orc_binom(L, ndown);
    bits_t *us = enumerate_strings(L, nup, Du);
    bits_t *ds = enumerate_strings(L, ndown, Dd);
    int64_t *bt = make_binom_tab();
#pragma omp parallel
    {
        rdm_t R;
        rdm_bind(&R, L, P.buf + (size_t)thread_id() * P.sz);
#pragma omp for schedule(dynamic, 1)
        for (int64_t ia = 0; ia < Du; ++ia) {
            const bits_t u1 = us[ia];
            for (int64_t ib = 0; ib < Dd; ++ib) {
                const bits_t d1 = ds[ib];
                const double cI = c[ia * Dd + ib];
                fill_diagonal(&R, u1, d1, cI * cI, 0);
                fill_diagonal(&R, u1, d1, cI * cI, 1);
                /* alpha singles and alpha-beta / alpha-alpha doubles with J_alpha > I_alpha */
                for (int j = 0; j < L; ++j) {
                    if (!(u1 & ((bits_t)1 << j))) continue;
                    for (int l = 0; l < L; ++l) {
                        if (u1 & ((bits_t)1 << l)) continue;
                        bits_t u2 = u1 ^ ((bits_t)1 << j) ^ ((bits_t)1 << l);
                        int64_t ja = string_rank(u2, bt, L);
                        if (ja <= ia) continue;
                        const double cj = c[ja * Dd + ib];
                        fill_one_dense(&R, u1, u2, d1, cI * cj, 0);
                        fill_one_dense(&R, u1, u2, d1, cI * cj, 2);
                        for (int m = 0; m < L; ++m) {
                            if (!(d1 & ((bits_t)1 << m))) continue;
                            for (int w = 0; w < L; ++w) {
                                if (d1 & ((bits_t)1 << w)) continue;
                                bits_t d2 = d1 ^ ((bits_t)1 << m) ^ ((bits_t)1 << w);
                                int64_t jb = string_rank(d2, bt, L);
                                fill_two_ud(&R, u1, u2, d1, d2, cI * c[ja * Dd + jb]);
                            }
                        }
                    }
                }
                for (int j = 0; j < L; ++j) {
                    if (!(u1 & ((bits_t)1 << j))) continue;
                    for (int j2 = j + 1; j2 < L; ++j2) {
                        if (!(u1 & ((bits_t)1 << j2))) continue;
                        for (int l = 0; l < L; ++l) {
                            if (u1 & ((bits_t)1 << l)) continue;
                            for (int l2 = l + 1; l2 < L; ++l2) {
                                if (u1 & ((bits_t)1 << l2)) continue;
                                bits_t u2 = u1 ^ ((bits_t)1 << j) ^ ((bits_t)1 << j2) ^ ((bits_t)1 << l) ^
                                            ((bits_t)1 << l2);
                                int64_t ja = string_rank(u2, bt, L);
                                if (ja <= ia) continue;
                                fill_two_dense(&R, u1, u2, cI * c[ja * Dd + ib], 0);
                            }
                        }
                    }
                }
                /* beta singles and beta-beta doubles with J_beta > I_beta (alpha equal) */
                for (int j = 0; j < L; ++j) {
                    if (!(d1 & ((bits_t)1 << j))) continue;
                    for (int l = 0; l < L; ++l) {
                        if (d1 & ((bits_t)1 << l)) continue;
                        bits_t d2 = d1 ^ ((bits_t)1 << j) ^ ((bits_t)1 << l);
                        int64_t jb = string_rank(d2, bt, L);
                        if (jb <= ib) continue;
                        const double cj = c[ia * Dd + jb];
                        fill_one_dense(&R, d1, d2, u1, cI * cj, 1);
                        fill_one_dense(&R, d1, d2, u1, cI * cj, 3);
                    }
                }
                for (int j = 0; j < L; ++j) {
                    if (!(d1 & ((bits_t)1 << j))) continue;
                    for (int j2 = j + 1; j2 < L; ++j2) {
                        if (!(d1 & ((bits_t)1 << j2))) continue;
                        for (int l = 0; l < L; ++l) {
                            if (d1 & ((bits_t)1 << l)) continue;
                            for (int l2 = l + 1; l2 < L; ++l2) {
                                if (d1 & ((bits_t)1 << l2)) continue;
                                bits_t d2 = d1 ^ ((bits_t)1 << j) ^ ((bits_t)1 << j2) ^ ((bits_t)1 << l) ^
                                            ((bits_t)1 << l2);
                                int64_t jb = string_rank(d2, bt, L);
                                if (jb <= ib) continue;
                                fill_two_dense(&R, d1, d2, cI * c[ia * Dd + jb], 2);
                            }
                        }
                    }
                }
            }
        }
    }
    free(us);
    free(ds);
    free(bt);
    pool_reduce(&P, L, rdm1, aa, ab, bb);
    return 0;
}

/* Rows [r0, r1) of the upper CRS, built with the same row generator as
 * orc_build_upper (bounded samples for the CPU baseline). With col == NULL
 * only counts[0..r1-r0) is filled; otherwise counts must hold the prefix
 * offsets (r1-r0+1 entries, counts[0] = 0) and col/val are filled. Rows are
 * spread over OpenMP threads. Returns the number of stored elements. */
int64_t orc_build_rows(int method, int L, int nup, int ndown, const double *h, const double *eri, int64_t r0,
                       int64_t r1, int64_t *counts, uint32_t *col, double *val) {
    if (L < 1 || L > 62 || r1 < r0) return -1;
    ham_t H = {L, nup, ndown, h, eri, (size_t)L, (size_t)L * L, (size_t)L * L * L};
    int64_t *bt = make_binom_tab();
    const int64_t Du = orc_binom(L, nup), Dd = (method == ORC_DOCI) ? 1 : orc_binom(L, ndown);
    bits_t *us = enumerate_strings(L, nup, Du);
    bits_t *ds = (method == ORC_DOCI) ? NULL : enumerate_strings(L, ndown, Dd);
    const int64_t sa = (int64_t)nup * (L - nup), sb = (int64_t)ndown * (L - ndown);
    const int64_t wmax = 2 + sa + sb + sa * sb + orc_binom(nup, 2) * orc_binom(L - nup, 2) +
                         orc_binom(ndown, 2) * orc_binom(L - ndown, 2);
    int64_t total = 0;
#pragma omp parallel reduction(+ : total)
    {
        rowbuf_t r;
        r.col = (uint32_t *)malloc((size_t)wmax * sizeof(uint32_t));
        r.val = (double *)malloc((size_t)wmax * sizeof(double));
#pragma omp for schedule(dynamic, 16)
        for (int64_t rr = r0; rr < r1; ++rr) {
            if (method == ORC_DOCI) {
                doci_row(&H, bt, us[rr], (long)rr, &r);
            } else {
                const int64_t i = rr / Dd, k = rr % Dd;
                fci_row(&H, bt, us[i], ds[k], (long)i, (long)k, (long)Dd, &r);
            }
            total += r.n;
            if (col == NULL) {
                counts[rr - r0] = r.n;
            } else {
                memcpy(col + counts[rr - r0], r.col, (size_t)r.n * sizeof(uint32_t));
                memcpy(val + counts[rr - r0], r.val, (size_t)r.n * sizeof(double));
            }
        }
        free(r.col);
        free(r.val);
    }
    free(us);
    free(ds);
    free(bt);
    return total;
}

/* The reference serial symmetric matvec restricted to rows [r0, r0+nrows) of
 * the upper CRS (local row pointers), accumulating into full-length y. */
void orc_sym_mvprod_rows(int64_t r0, int64_t nrows, const int64_t *row, const uint32_t *col, const double *val,
                         const double *x, double *y) {
    for (int64_t i = 0; i < nrows; ++i) {
        const int64_t gi = r0 + i;
        for (int64_t k = row[i]; k < row[i + 1]; ++k) {
            y[gi] += val[k] * x[col[k]];
            if ((uint32_t)gi != col[k]) y[col[k]] += val[k] * x[gi];
        }
    }
}

/* ---- determinant lists: FCI_File::construct_CI_matrix (CIMethod.cpp:890-914) with
 *      get_ham_element (CIMethod.cpp:459-487), strings of up to 128 orbitals ---- */
typedef unsigned __int128 wide_t;

static inline int popc_w(wide_t x) {
    return __builtin_popcountll((uint64_t)x) + __builtin_popcountll((uint64_t)(x >> 64));
}
static inline int ctz_w(wide_t x) {
    const uint64_t lo = (uint64_t)x;
    return lo ? __builtin_ctzll(lo) : 64 + __builtin_ctzll((uint64_t)(x >> 64));
}
static inline int get_orbs_w(wide_t s, int *o) {
    int n = 0;
    while (s) {
        o[n++] = ctz_w(s);
        s &= s - 1;
    }
    return n;
}
static inline int nstacked_w(int o0, int o1, wide_t up) {
    int lo = o0 < o1 ? o0 : o1, hi = o0 < o1 ? o1 : o0;
    int sum = 0;
    for (int i = lo; i < hi; ++i)
        if ((up >> i) & 1) ++sum;
    return sum;
}
static inline void arrange_w(int *orbs, int num, wide_t up1) {
    int re[4];
    int a = 0, b = (num == 4) ? 2 : 1;
    for (int i = 0; i < num; ++i) {
        if ((up1 >> orbs[i]) & 1)
            re[a++] = orbs[i];
        else
            re[b++] = orbs[i];
    }
    for (int i = 0; i < num; ++i) orbs[i] = re[i];
}
static double diag_one_w(const ham_t *H, wide_t s) {
    int o[128];
    const int n = get_orbs_w(s, o);
    return diag_one(H, o, n);
}
static double diagonal_w(const ham_t *H, wide_t up, wide_t dn) {
    int ou[128] = {0}, od[128] = {0};
    const int nu = get_orbs_w(up, ou), nd = get_orbs_w(dn, od);
    double tot = diag_one(H, ou, nu);
    tot += diag_one(H, od, nd);
    double mix = 0;
    for (int k = 0; k < nu; ++k)
        for (int l = 0; l < nd; ++l) mix += V(H, ou[k], od[l], ou[k], od[l]);
    tot += mix;
    (void)diag_one_w;
    return tot;
}
static double one_diff_w(const ham_t *H, wide_t s1, wide_t s2, wide_t other) {
    int orbs[128], com[128], oth[128];
    get_orbs_w(s1 ^ s2, orbs);
    double e = T(H, orbs[0], orbs[1]);
    const int nc = get_orbs_w(s1 & s2, com);
    for (int z = 0; z < nc; ++z)
        e += V(H, orbs[0], com[z], orbs[1], com[z]) - V(H, orbs[0], com[z], com[z], orbs[1]);
    const int diff = nstacked_w(orbs[0], orbs[1], s1 & s2);
    const int no = get_orbs_w(other, oth);
    for (int z = 0; z < no; ++z) e += V(H, orbs[0], oth[z], orbs[1], oth[z]);
    if (diff % 2 != 0) e *= -1;
    return e;
}
static double two_same_w(const ham_t *H, wide_t s1, wide_t s2) {
    int o[128];
    get_orbs_w(s1 ^ s2, o);
    arrange_w(o, 4, s1);
    const wide_t c = s1 & s2;
    const int diff = nstacked_w(o[0], o[1], c) + nstacked_w(o[2], o[3], c);
    double e = V(H, o[0], o[1], o[2], o[3]) - V(H, o[0], o[1], o[3], o[2]);
    if (diff % 2 != 0) e *= -1;
    return e;
}
static double two_ab_w(const ham_t *H, wide_t u1, wide_t u2, wide_t d1, wide_t d2) {
    int a[128], b[128];
    get_orbs_w(u1 ^ u2, a);
    get_orbs_w(d1 ^ d2, b);
    arrange_w(a, 2, u1);
    arrange_w(b, 2, d1);
    const int diff = nstacked_w(a[0], a[1], u1 & u2) + nstacked_w(b[0], b[1], d1 & d2);
    double e = V(H, a[0], b[0], a[1], b[1]);
    if (diff % 2 != 0) e *= -1;
    return e;
}
static double ham_element_w(const ham_t *H, wide_t up1, wide_t down1, wide_t up2, wide_t down2) {
    const int nu = popc_w(up1 ^ up2), nd = popc_w(down1 ^ down2);
    if (nd > 4 || nu > 4) return 0;
    if (nu == 4 && nd == 0) return two_same_w(H, up1, up2);
    if (nu == 2) {
        if (nd == 0) return one_diff_w(H, up1, up2, down1);
        if (nd == 2) return two_ab_w(H, up1, up2, down1, down2);
        return 0;
    }
    if (nd == 4 && nu == 0) return two_same_w(H, down1, down2);
    if (nd == 2 && nu == 0) return one_diff_w(H, down1, down2, up1);
    if (nd == 0 && nu == 0) return diagonal_w(H, up1, down1);
    return 0;
}

int orc_build_dets(int L, int nup, int ndown, const double *h, const double *eri, int64_t ndet, int words,
                   const uint64_t *up, const uint64_t *down, int64_t *row, uint32_t *col, double *val) {
    if (L < 1 || L > 128 || ndet < 1 || (words != 1 && words != 2)) return 1;
    ham_t H = {L, nup, ndown, h, eri, (size_t)L, (size_t)L * L, (size_t)L * L * L};
    wide_t *us = (wide_t *)malloc((size_t)ndet * sizeof(wide_t));
    wide_t *ds = (wide_t *)malloc((size_t)ndet * sizeof(wide_t));
    for (int64_t i = 0; i < ndet; ++i) {
        us[i] = up[i * words];
        ds[i] = down[i * words];
        if (words == 2) {
            us[i] |= (wide_t)up[i * words + 1] << 64;
            ds[i] |= (wide_t)down[i * words + 1] << 64;
        }
    }
    const int fill = (col != NULL);
#pragma omp parallel
    {
        rowbuf_t r;
        r.col = (uint32_t *)malloc((size_t)ndet * sizeof(uint32_t));
        r.val = (double *)malloc((size_t)ndet * sizeof(double));
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < ndet; ++i) {
            r.n = 0;
            for (int64_t j = i; j < ndet; ++j) push_row(&r, (uint32_t)j, ham_element_w(&H, us[i], ds[i], us[j], ds[j]), 1);
            if (!fill) {
                row[i + 1] = r.n;
            } else {
                memcpy(col + row[i], r.col, (size_t)r.n * sizeof(uint32_t));
                memcpy(val + row[i], r.val, (size_t)r.n * sizeof(double));
            }
        }
        free(r.col);
        free(r.val);
    }
    if (!fill) {
        row[0] = 0;
        for (int64_t i = 0; i < ndet; ++i) row[i + 1] += row[i];
    }
    free(us);
    free(ds);
    return 0;
}

/* DensFILE::construct_CI_one_dens / construct_CI_two_dens (CIDens.cpp:1468-1529): every
 * pair i <= j of a determinant list (64-bit strings) through fill_density_matrix_one /
 * fill_density_matrix with contr = c_i c_j. Outputs as orc_rdm_pairs. */
int orc_rdm_dets(int L, int ndet, const uint64_t *up, const uint64_t *down, const double *c, double *rdm1,
                 double *aa, double *ab, double *bb) {
    if (L < 2 || L > 62 || ndet < 1) return 1;
    rdm_pool_t P;
    pool_init(&P, L);
#pragma omp parallel
    {
        rdm_t R;
        rdm_bind(&R, L, P.buf + (size_t)thread_id() * P.sz);
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < ndet; ++i)
            for (int j = i; j < ndet; ++j) {
                const double contr = c[i] * c[j];
                fill_pair_one(&R, up[i], down[i], up[j], down[j], contr);
                fill_pair_two(&R, up[i], down[i], up[j], down[j], contr);
            }
    }
    pool_reduce(&P, L, rdm1, aa, ab, bb);
    return 0;
}

