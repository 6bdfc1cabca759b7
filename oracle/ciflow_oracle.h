/* CPU restatement of the CIFlow lowest-eigenpair CI path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker the GPU path is
 * compared against; it is loaded by tests/, by __graft_entry__.smoke() and by
 * the CPU-baseline leg of bench.py, never by the product library.
 *
 * Integrals: h is L*L row-major; eri is chemist (pq|rs), L^4 row-major. The
 * physics element the reference uses is V(i,j,k,l) = <ij|kl> = (ik|jl).
 * Bitstrings are 64-bit, so L <= 63 (determinant lists: 128-bit, L <= 128).
 * nup must equal ndown for DOCI.
 */
#ifndef CIGPU_ORACLE_H
#define CIGPU_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FCI = 0, ORC_DOCI = 1 };

/* Exact binomial coefficient C(n,k) (0 when k<0 or k>n). */
int64_t orc_binom(int n, int k);
/* Dimension of the determinant space. */
int64_t orc_dim(int method, int L, int nup, int ndown);

/* Upper-triangle CRS in the reference layout (SparseMatrix_CRS_Sym filled by
 * FCI/DOCI::construct_CI_matrix). Two calls: with col == NULL it only fills
 * row[0..dim] (row pointers, 64-bit here); then with col/val of row[dim]
 * entries it fills the pattern and values. */
int orc_build_upper(int method, int L, int nup, int ndown, const double *h, const double *eri,
                    int64_t *row, uint32_t *col, double *val);

/* y = (U + U^T - D) x from the upper CRS, the serial scatter of
 * SparseMatrix_CRS_Sym::mvprod. */
void orc_sym_mvprod(int64_t n, const int64_t *row, const uint32_t *col, const double *val, const double *x,
                    double *y);
/* The same product with OpenMP over rows of the full matrix, for large oracle solves:
 * y = U x via rows plus U^T x via per-thread scatter buffers. */
void orc_sym_mvprod_omp(int64_t n, const int64_t *row, const uint32_t *col, const double *val, const double *x,
                        double *y);

/* RDMs of the state c, with the reference CIDens conventions. Outputs:
 *   rdm1 [2][L][L]            get_one_rdm(spin,i,j)
 *   aa, bb [np][np]           get_two_rdm(0|2,p,q,r,s) for p<q, r<s, np = L(L-1)/2,
 *                             pair index p*L+q-(p+1)(p+2)/2
 *   ab [L*L][L*L]             get_two_rdm(1,p,q,r,s)
 * orc_rdm_pairs follows DensFCI/DensDOCI literally (O(dim^2) pair loop for FCI);
 * orc_rdm_excitations enumerates only connected pairs (same contributions). */
int orc_rdm_pairs(int method, int L, int nup, int ndown, const double *c, double *rdm1, double *aa, double *ab,
                  double *bb);
int orc_rdm_excitations(int method, int L, int nup, int ndown, const double *c, double *rdm1, double *aa,
                        double *ab, double *bb);

/* Upper-triangle CRS of a determinant list in list order (FCI_File::construct_CI_matrix
 * with get_ham_element): strings of `words` 64-bit words (L <= 128). Two calls as
 * orc_build_upper. */
int orc_build_dets(int L, int nup, int ndown, const double *h, const double *eri, int64_t ndet, int words,
                   const uint64_t *up, const uint64_t *down, int64_t *row, uint32_t *col, double *val);

/* RDMs of a determinant list's state (DensFILE: every pair i <= j, 64-bit strings). */
int orc_rdm_dets(int L, int ndet, const uint64_t *up, const uint64_t *down, const double *c, double *rdm1,
                 double *aa, double *ab, double *bb);

/* Bounded samples for the CPU baseline: rows [r0, r1) of the upper CRS (see the .c file). */
int64_t orc_build_rows(int method, int L, int nup, int ndown, const double *h, const double *eri, int64_t r0,
                       int64_t r1, int64_t *counts, uint32_t *col, double *val);
void orc_sym_mvprod_rows(int64_t r0, int64_t nrows, const int64_t *row, const uint32_t *col, const double *val,
                         const double *x, double *y);

#ifdef __cplusplus
}
#endif
#endif
