/* cigpu: GB300-native lowest-eigenpair CI core, C ABI.
 *
 * This is the drop-in boundary for CIFlow's lowest-eigenpair path. Each entry
 * point names the reference interface (file:line in the CIFlow tree) whose job
 * it takes over. All compute runs in hand-written sm_103a CUDA kernels; there is
 * no CPU fallback: without a usable GPU every compute call returns
 * CIGPU_ECUDA.
 *
 * Conventions
 *  - Every call returns an int status (CIGPU_OK == 0). Nothing exits or traps.
 *  - Handles own their device memory; the caller owns every host buffer.
 *  - Integrals: h is L*L row-major and symmetric; eri is the chemist-notation
 *    tensor (pq|rs), L^4 row-major, 8-fold symmetric. The physics element the
 *    reference uses is V(i,j,k,l) = <ij|kl> = (ik|jl).
 *  - Determinants are ordered like CIFlow: row = I_alpha * D_beta + I_beta, each
 *    string ranked in colex (Gosper) order; DOCI rows are pair strings.
 *  - Energies returned by the solvers include Econst.
 *  - A handle is used by one host thread at a time; distinct handles may be
 *    used concurrently. The server object is internally synchronised.
 */
#ifndef CIGPU_H
#define CIGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CIGPU_ABI_VERSION 1

typedef struct cigpu_ham cigpu_ham;
typedef struct cigpu_crs cigpu_crs;
typedef struct cigpu_server cigpu_server;
/* A cudaStream_t passed as an opaque pointer; NULL selects the handle's own stream. */
typedef void *cigpu_stream;

enum cigpu_status {
    CIGPU_OK = 0,
    CIGPU_EINVAL = 22,     /* bad argument, size or non-symmetric / non-finite integrals */
    CIGPU_ENOMEM = 12,     /* device or host allocation failed, or HBM budget exceeded */
    CIGPU_EAGAIN = 11,     /* server queue full: retry later */
    CIGPU_ECANCELED = 125, /* request cancelled */
    CIGPU_ETIMEDOUT = 110, /* a bounded wait expired */
    CIGPU_ENOTSUP = 95,    /* combination not supported (e.g. L > 63) */
    CIGPU_ENOCONV = 200,   /* eigensolver hit its matvec limit before the tolerance */
    CIGPU_ECUDA = 201,     /* CUDA error or no usable GPU */
    CIGPU_ENOTFOUND = 202  /* unknown request id */
};

/* CIGPU_DETS: a CRS made by cigpu_build_dets from a determinant list (FCI_File / CI_Big). */
enum cigpu_method { CIGPU_FCI = 0, CIGPU_DOCI = 1, CIGPU_DETS = 2 };
/* FP64: FP64 CRS values, FP64 Krylov vectors, FP64 matvec.
 * MIXED: FP32 CRS values and FP32 Krylov vectors with FP32 row accumulation;
 *        FP64 orthogonalisation coefficients, recurrence, projected eigensolve,
 *        Rayleigh quotient and residual (FP64 matvec) with residual-correction
 *        restarts. */
enum cigpu_precision { CIGPU_FP64 = 0, CIGPU_MIXED = 1 };

typedef struct {
    double e0;               /* lowest eigenvalue including Econst */
    double residual;         /* ||H c - E c||_2 with ||c|| = 1, computed with an FP64 matvec */
    double error_bound;      /* residual^2 / gap estimate (bound on |E - E_exact|) */
    double gap;              /* estimated gap to the next Ritz value */
    int64_t matvecs_fp64;    /* FP64 matrix-vector products */
    int64_t matvecs_fp32;    /* FP32 matrix-vector products */
    int32_t restarts;        /* thick restarts (FP64); MIXED: folds that kept the previous Ritz direction */
    int32_t corrections;     /* FP64 residual-correction cycles (MIXED) */
    int32_t converged;       /* 1 when residual <= tol */
    int32_t precision;       /* cigpu_precision the solve ran in (cigpu_solve_batch may
                                run a problem in FP64 although MIXED was requested) */
    double seconds;          /* wall time of the solve */
} cigpu_solve_info;

/* ---- library ---- */
int cigpu_get_version(void);
const char *cigpu_strerror(int status);
/* Number of CUDA devices visible (0 without a GPU; returns CIGPU_ECUDA then). */
int cigpu_device_count(int *count);
/* Kernels this library launched since load (for launch accounting). */
int64_t cigpu_kernel_launches(void);
/* The checked build (libcigpu_checked.so, compiled with -DCIGPU_CHECKED) tests every
 * index its kernels derive from stored data before using it (matvec columns, CRS row
 * bounds, DOCI hop ranks, RDM pair / term / excitation indices), skips a failing
 * access and records the first violation in a per-device error word: code << 56 |
 * index (codes: 1 column, 2 row bounds, 3 hop rank, 4 RDM pair, 5 RDM term, 6 RDM
 * excitation). The reference asserts the same bounds in its accessors
 * (matrix.cpp:676-677, SparseMatrix_CRS.cpp:691-693) and exits on a failure.
 * cigpu_checked_build returns 1 in the checked build, 0 otherwise. cigpu_check_word
 * waits for the device and reads (reset != 0: then clears) the current device's
 * word (0: no violation); CIGPU_ENOTSUP in the regular build. */
int cigpu_checked_build(void);
int cigpu_check_word(uint64_t *word, int reset);

/* ---- Hamiltonian: replaces Hamiltonian(L, nGroup=0, nup, ndown, Econst) plus
 * setTmat/setVmat (Hamiltonian.cpp:77-113, 255-320) and the getTmat/getVmat
 * lookups every matrix element goes through (FourIndex.cpp:175-315). The tensors
 * are copied to the device as dense tables. ---- */
int cigpu_ham_create(int L, int nup, int ndown, double econst, const double *h, const double *eri,
                     cigpu_ham **out);
/* (L <= 128; FCI/DOCI builds, rotations and the server need L <= 63, determinant lists take up to 128.) */
int cigpu_ham_destroy(cigpu_ham *ham);
/* ---- orbital rotation: replaces OrbitalTransform::fillHamCI and rotate_old_to_new
 * (OrbitalTransform.cpp:64-170). Creates a new Hamiltonian with the integrals of
 * `base` rotated on the device by the orthogonal L x L matrix U (row-major,
 * U[a*L + p]): h'_ab = sum U_ap U_bq h_pq, (ab|cd)' = sum U_ap U_bq U_cr U_ds (pq|rs),
 * made exactly 8-fold symmetric. Runs on `stream` (NULL: a private stream) and
 * returns when done. CIGPU_EINVAL if U is not orthogonal to 1e-10. ---- */
int cigpu_ham_rotate(const cigpu_ham *base, const double *U, cigpu_stream stream, cigpu_ham **out);
/* Integrals held by a Hamiltonian (h: L*L, eri: L^4 chemist; either may be NULL),
 * e.g. after cigpu_ham_rotate; getTmat/getVmat (Hamiltonian.cpp:255-320). */
int cigpu_ham_export(const cigpu_ham *ham, double *h, double *eri);
/* U = exp(X) for an antisymmetric L x L generator X (row-major), the unitary of
 * UnitaryMatrix::updateUnitary (UnitaryMatrix.cpp:229-290). Host computation. */
int cigpu_unitary_exp(int L, const double *X, double *U);

/* ---- CRS build: replaces new FCI(ham) / new DOCI(ham), i.e.
 * CIMethod::build_parallel + FCI::construct_CI_matrix / DOCI::construct_CI_matrix
 * (CIMethod.cpp:489-561, 749-888, 611-660) filling SparseMatrix_CRS_Sym.
 * The device keeps the full symmetric matrix (both triangles, columns ascending);
 * its upper triangle is CIFlow's CRS exactly (same 1e-14 drop threshold).
 * The ham handle is borrowed and must outlive the CRS. A MIXED FCI build whose
 * FP32 products come from the sigma operator (cigpu_crs_fp32_product) returns
 * before its FP64 values and row counts are complete: they are made on the
 * handle's own side stream while a solve starts, the FP64 products wait for them
 * on the device, and cigpu_crs_dims (when asked for the nonzero counts), the
 * exports and cigpu_crs_destroy wait for them on the host. ---- */
int cigpu_build(cigpu_ham *ham, int method, int precision, cigpu_stream stream, cigpu_crs **out);
int cigpu_crs_destroy(cigpu_crs *crs);
/* dim only: no wait; nnz_upper / nnz_full: after the build's deferred part. */
int cigpu_crs_dims(const cigpu_crs *crs, int64_t *dim, int64_t *nnz_upper, int64_t *nnz_full);
/* Device storage of the matrix (no reference counterpart; reported with matvec
 * measurements). CIGPU_LAYOUT_CRS: full symmetric CRS, stored = nnz_full values
 * with a 4-byte column each. CIGPU_LAYOUT_SLOTS (FCI): values only (FP32 hi + lo
 * for MIXED, FP64 for FP64 and for MIXED with the sigma FP32 product), every structural slot of every row (zeros included,
 * rows padded to tiles of 64 beta strings), stored = that slot count; columns are
 * regenerated from the string tables. With CIGPU_SLOTS64=compact in the environment
 * (read at each build) FP64 tiles leave out each row's alpha-single x beta-single
 * block, which the FP64 product forms from the integrals (same results bit for bit;
 * 3.4x fewer values at 12 orbitals 6a6b, a 40% slower product), and stored counts
 * the values kept. CIGPU_LAYOUT_PAIRS (DOCI): no stored matrix,
 * stored = 0; every matvec generates the pair hops from the pair strings and the
 * L x L table K_jk = (jk|jk). CIGPU_LAYOUT_ONTHEFLY: determinant lists without a
 * stored matrix. The explicit CRS of every layout is generated for the exports. */
enum { CIGPU_LAYOUT_CRS = 0, CIGPU_LAYOUT_SLOTS = 1, CIGPU_LAYOUT_ONTHEFLY = 2, CIGPU_LAYOUT_PAIRS = 3 };
int cigpu_crs_layout(const cigpu_crs *crs, int *layout, int64_t *stored);
/* The FP32 product of a MIXED matrix (no reference counterpart; reported with
 * matvec measurements). CIGPU_FP32_STORED: the stored FP32 values (slot tiles,
 * CRS) or the DOCI pair hops. CIGPU_FP32_SIGMA (FCI): a direct-CI sigma vector
 * from a factorisation (pq|rs) = sum_k s_k F^k_pq F^k_rs, rank = the factors kept,
 * padded = the rank the kernels run (a multiple of 16); the FP64 products use the
 * stored matrix. rank and padded are 0 for the stored product. FP64 matrices
 * report CIGPU_FP32_STORED. The environment variable CIGPU_FP32_PRODUCT, read at
 * each build, selects "slots" or "sigma"; by default the sigma product is taken
 * where its 32 x 32 string tiles outnumber the SMs. */
enum { CIGPU_FP32_STORED = 0, CIGPU_FP32_SIGMA = 1 };
int cigpu_crs_fp32_product(const cigpu_crs *crs, int *kind, int *rank, int *padded);
/* Upper triangle in the reference layout (SparseMatrix_CRS::row/col/data,
 * SparseMatrix_CRS.h:107-111): row[dim+1], col[nnz_upper], val[nnz_upper]. Host buffers. */
int cigpu_crs_export_upper(cigpu_crs *crs, uint32_t *row, uint32_t *col, double *val);
/* Full matrix as stored on the device: row[dim+1] (64-bit), col/val[nnz_full]. Host buffers. */
int cigpu_crs_export_full(cigpu_crs *crs, int64_t *row, uint32_t *col, double *val);

/* ---- matvec: replaces SparseMatrix_CRS_Sym::mvprod(const double*, double*)
 * (SparseMatrix_CRS.cpp:700-723; virtual at SparseMatrix_CRS.h:126).
 * Host buffers x, y of length dim; FP64 arithmetic (for a MIXED CRS the FP64
 * product uses the stored FP32 split of each value, v = hi + lo, exact to
 * 2^-48 relative). The copies and the product run on `stream` (NULL: the CRS
 * stream); the call returns when y is filled. ---- */
int cigpu_mvprod(cigpu_crs *crs, const double *x, double *y, cigpu_stream stream);
/* Device-buffer form on the given stream. dtype 0: FP64 x/y (FP64 matvec);
 * dtype 1: FP32 x/y (FP32 values, FP32 accumulation; MIXED CRS only). */
int cigpu_mvprod_device(cigpu_crs *crs, const void *x, void *y, int dtype, cigpu_stream stream);

/* ---- eigensolver: replaces CIMethod::solve + SparseMatrix_CRS::arpackDiagonalize
 * (CIMethod.cpp:241-264, SparseMatrix_CRS.cpp:360-481) for neig = 1. GPU-resident
 * thick-restart Lanczos with full orthogonalisation (basis 42, like ARPACK's ncv).
 * tol: FP64 residual norm target. max_matvec: limit (0 = 3*dim like iparam[2]).
 * c0: optional start vector (host, dim; NULL = seeded random). c_out: optional
 * host buffer (dim) for the normalised eigenvector. Unlike the reference, the
 * CRS stays resident after the solve (the reference frees it, CIMethod.cpp:262). ---- */
int cigpu_solve(cigpu_crs *crs, double tol, int64_t max_matvec, const double *c0, double *c_out,
                cigpu_solve_info *info);

/* ---- RDMs: replaces CIMethod::construct_density / CIDens::construct_density with
 * DensFCI / DensDOCI (CIMethod.cpp:161-171, CIDens.cpp:323-334, 1073-1224, 1530-1631).
 * c: host, dim (normalised state). Outputs (host, any may be NULL to skip):
 *   rdm1 [2][L][L]         = CIDens::get_one_rdm(spin, i, j)
 *   rdm2_aa, rdm2_bb [np][np], np = L(L-1)/2, pair(p<q) = p*L+q-(p+1)(p+2)/2
 *                          = get_two_rdm(0|2, p, q, r, s) for p<q, r<s
 *   rdm2_ab [L*L][L*L]     = get_two_rdm(1, p, q, r, s) at (p*L+q, r*L+s) ---- */
int cigpu_rdm(cigpu_crs *crs, const double *c, double *rdm1, double *rdm2_aa, double *rdm2_ab, double *rdm2_bb);

/* ---- DOCI RDMs without device allocation. No counterpart in the reference.
 * For callers that cannot allocate device memory on their request path (a host
 * framework that owns all device memory through its own fixed pool, or a
 * latency-bound loop that cannot afford the device synchronisation cudaMalloc
 * implies): the block partial sums live in a fixed 4 MiB array inside the
 * library, so this call allocates nothing. crs must be a DOCI CRS with L <= 32
 * (CIGPU_ENOTSUP otherwise). c (dim) and the outputs, laid out as in cigpu_rdm,
 * are DEVICE buffers; the work is queued on `stream` (NULL: the CRS stream) and
 * the call returns without waiting. Call it with the CRS's device current
 * (CIGPU_EINVAL otherwise). The first call on a device looks up the array's
 * device address and keeps it for the life of the process (it does not survive
 * a cudaDeviceReset); make that first call before any stream capture. Calls
 * share the array: calls that overlap on the GPU race, so serialise them. ---- */
int cigpu_rdm_doci_noalloc(cigpu_crs *crs, const double *c, double *rdm1, double *rdm2_aa, double *rdm2_ab,
                           double *rdm2_bb, cigpu_stream stream);

/* ---- serving: continuous batching of independent solves (the served analogue of
 * the set_ham -> solve loop of the orbital optimisers, SimulatedAnnealing.cpp:72-86,
 * 130-134; CIMethod::set_ham CIMethod.cpp:117-126). Requests are admitted as
 * device memory (the HBM budget) and slots free up; admitted requests run
 * concurrently on separate streams (for many small problems known up front,
 * cigpu_solve_batch below packs them into shared launches). ---- */
typedef struct {
    int32_t L, nup, ndown;
    int32_t method;      /* cigpu_method */
    int32_t precision;   /* cigpu_precision */
    int32_t want_rdm;    /* 1: also compute the 1-RDM */
    double econst;
    double tol;          /* FP64 residual target */
    const double *h;     /* copied at submit */
    const double *eri;   /* copied at submit */
    const double *c0;    /* optional warm start (dim), copied at submit */
    const double *rot;   /* optional L x L orbital rotation U applied to (h, eri) on the
                            device before the build (cigpu_ham_rotate); copied at submit */
} cigpu_request;

typedef struct {
    int32_t status;      /* CIGPU_OK, CIGPU_ENOCONV, CIGPU_ECANCELED, ... */
    int32_t done;        /* 1 when finished */
    int64_t dim;
    cigpu_solve_info info;
    double queued_s;     /* submit -> admission */
    double latency_s;    /* submit -> completion */
} cigpu_result;

int cigpu_server_create(int device, size_t hbm_budget_bytes, int max_inflight, int max_queue,
                        cigpu_server **out);
/* Returns CIGPU_EAGAIN when the queue is full, CIGPU_ENOMEM when the request can
 * never fit the budget, CIGPU_EINVAL on bad input. */
int cigpu_server_submit(cigpu_server *srv, const cigpu_request *req, uint64_t *id);
/* Waits up to wait_ms (0 = poll, <0 = until done) for request id. c_out (dim)
 * and rdm1 ([2][L][L]) are optional host buffers filled when done. The request
 * is released after a completed poll. */
int cigpu_server_poll(cigpu_server *srv, uint64_t id, int wait_ms, cigpu_result *out, double *c_out,
                      double *rdm1);
int cigpu_server_cancel(cigpu_server *srv, uint64_t id);
int cigpu_server_stats(cigpu_server *srv, int64_t *admitted, int64_t *completed, int64_t *inflight,
                       size_t *hbm_in_use);
int cigpu_server_destroy(cigpu_server *srv);

/* ---- batched solves: many independent lowest-eigenpair problems in one call.
 * Replaces a loop of CIMethod::solve over Hamiltonians (CIMethod.cpp:241-264), as
 * the orbital optimisers run it (SimulatedAnnealing.cpp:72-86). Problems with at
 * most max_batched_dim determinants (0: 65536) are built as FP64 CRS matrices and
 * solved together by a lockstep FP64 Lanczos whose steps are CUDA-graph launches
 * serving every problem (their precision field is not used); larger problems are
 * solved one by one with their requested precision on a stream of their own,
 * overlapping the batched ones. Request fields as for the server (want_rdm and c0 of batched problems
 * are ignored). Outputs per request (each optional): e0, info, status (CIGPU_OK,
 * CIGPU_ENOCONV, or the build error). Returns CIGPU_EINVAL for a malformed
 * request before any work, else the first build/solve error or CIGPU_OK. ---- */
typedef struct {
    int32_t batched;         /* problems solved in lockstep */
    int32_t individual;      /* problems above max_batched_dim */
    int32_t lanes, grid;     /* autotuned SpMV shape of the row class with most nonzeros (last batch) */
    int32_t steps;           /* Lanczos steps of the longest batch */
    int32_t graph_launches;  /* CUDA-graph launches (one per step of all problems) */
    int32_t tuned;           /* batches whose shape was timed now (not cached) */
    int32_t reserved;
    double seconds_build;    /* building the batched problems */
    double seconds;          /* the whole call */
} cigpu_batch_stats;
int cigpu_solve_batch(int count, const cigpu_request *req, int64_t max_batched_dim, double *e0,
                      cigpu_solve_info *info, int *status, cigpu_batch_stats *stats);

/* ---- determinant lists: replaces FCI_File (CIMethod.h:164-173, CIMethod.cpp:890-919)
 * and CI_Big (CIMethod.h:176-189, CIMethod.cpp:591-609, 928-1144) with
 * get_ham_element (CIMethod.cpp:459-487): a CI matrix over an arbitrary list of
 * determinants in list order. up/down: ndet strings of `words` 64-bit words each
 * (word 0 holds orbitals 0..63; words = 2 for L up to 128), each with the
 * Hamiltonian's nup / ndown electrons (CIGPU_EINVAL otherwise). storage:
 * CIGPU_DETS_CRS builds the CRS (its upper triangle is the reference's
 * SparseMatrix_CRS_Sym for the list, precision FP64 or MIXED);
 * CIGPU_DETS_ONTHEFLY stores no matrix (FP64 only): every matvec recomputes the
 * elements from the list, as CI_Big does for the part it does not keep. The CRS
 * handle works with cigpu_solve, cigpu_mvprod, (CRS storage) the exports, and
 * cigpu_rdm for L <= 64 (DensFILE, CIDens.cpp:1468-1529: every pair of the list
 * through the reference's fill rules; sums in 64-bit fixed point, bit-reproducible). ---- */
enum { CIGPU_DETS_CRS = 0, CIGPU_DETS_ONTHEFLY = 1 };
int cigpu_build_dets(cigpu_ham *ham, int64_t ndet, int words, const uint64_t *up, const uint64_t *down, int storage,
                     int precision, cigpu_stream stream, cigpu_crs **out);
/* CI_Big with its stored part (CI_Big::CI_Big and CI_Big::mvprod, CIMethod.cpp:591-609,
 * 943-984): the block of the matrix among the first `keep` determinants of the list
 * (0 <= keep <= ndet) is stored as a CRS; every matvec multiplies it and recomputes
 * each element outside it (rows or columns at or past `keep`). FP64 only. The
 * reference sizes keep from its CISIZE memory budget (numlines, CIMethod.cpp:596-598);
 * keep = 0 is CIGPU_DETS_ONTHEFLY, keep = ndet stores everything. cigpu_crs_dims
 * and cigpu_crs_layout report the stored block's elements. */
int cigpu_build_dets_partial(cigpu_ham *ham, int64_t ndet, int words, const uint64_t *up, const uint64_t *down,
                             int64_t keep, cigpu_stream stream, cigpu_crs **out);
/* Permutator_File::read_file (Permutator.cpp:179-224): a determinant file with one
 * "<up>|<down>" line per determinant (binary strings, orbital 0 rightmost; lines
 * holding '#' are skipped). Call with up/down NULL to count: *ndet = number of
 * determinants, *max_orbitals = longest string; then with arrays of capacity*words
 * words each. CIGPU_ENOTFOUND if the file cannot be opened, CIGPU_EINVAL on a
 * malformed line or a string longer than 64*words bits. Host code. */
int cigpu_dets_read(const char *path, int words, int64_t capacity, uint64_t *up, uint64_t *down, int64_t *ndet,
                    int *max_orbitals);

/* ---- on-disk formats (host code, no GPU needed) ----
 * cigpu_ham_read_psi4: Hamiltonian::read_file (Hamiltonian.cpp:707-885), the psi4
 * plugin's integral text dump: call with h == eri == NULL for L, nup, ndown, Econst
 * (and irreps[L] when given), then with h (L*L) and eri (L^4, chemist (pq|rs)) to
 * fill them; every listed element sets its symmetry partners, unlisted ones are 0.
 * Values are parsed as the reference parses them (the text after the indices
 * without the line's last character). Optional overlap / unitary sections are
 * skipped. hf_energy (optional) = the "HF Energy" trailer. CIGPU_ENOTFOUND /
 * CIGPU_EINVAL for a missing or malformed file.
 * cigpu_ham_write_psi4: Hamiltonian::save_file's format (Hamiltonian.cpp:646-705)
 * for point group C1, with 17 significant digits (exact round trip; the reference
 * writes 15) and each two-electron element once (p >= q, r >= s, pq >= rs). */
int cigpu_ham_read_psi4(const char *path, int *L, int *nup, int *ndown, double *econst, double *h, double *eri,
                        int *irreps, double *hf_energy);
int cigpu_ham_write_psi4(const char *path, int L, int nup, int ndown, double econst, const double *h,
                         const double *eri, double hf_energy);
/* The CI-vector text of the reference's output (OutputSingleFile::print_solutions +
 * OutputSFFCI / OutputSFDOCI / OutputSFFCI_File::print_ci_vec, Output.cpp:135-144,
 * 190-263): e0 (with Econst) and every coefficient with |c| >= threshold, with its
 * determinant's strings. method: CIGPU_FCI, CIGPU_DOCI (colex order) or CIGPU_DETS
 * (up/down: the list, `words` 64-bit words per string). Each DOCI line carries its
 * own pair string (the reference advances the string only on printed lines).
 * list_name (CIGPU_DETS, optional): the list's name in the header line. */
int cigpu_write_civec(const char *path, int method, int L, int nup, int ndown, int64_t dim, const double *c,
                      double e0, double econst, double threshold, const uint64_t *up, const uint64_t *down,
                      int words, const char *list_name);
/* The RDM text of CIMethod::print_one_rdm / print_two_rdm (CIMethod.cpp:184-195,
 * CIDens.cpp:978-1026) from arrays laid out as cigpu_rdm fills them; the 2-RDM part
 * is written when all three 2-RDM arrays are given. */
int cigpu_write_rdm(const char *path, int L, const double *rdm1, const double *rdm2_aa, const double *rdm2_ab,
                    const double *rdm2_bb);

/* Device memory a request of this shape needs (bytes), as used by admission. */
int cigpu_estimate_bytes(int L, int nup, int ndown, int method, int precision, size_t *bytes);

/* ---- Jacobi rotation of two orbitals: replaces OrbitalTransform::do_jacobi_rotation
 * (OrbitalTransform.cpp:278-414) for point group C1. Creates a new Hamiltonian whose
 * orbitals k and l are k' = cos(theta) k - sin(theta) l, l' = sin(theta) k + cos(theta) l
 * (the rows of the unitary, UnitaryMatrix::jacobi_rotation, UnitaryMatrix.cpp:186-207),
 * all other orbitals unchanged; the result is exactly 8-fold symmetric. Runs on
 * `stream` (NULL: a private stream) and returns when done. ---- */
int cigpu_ham_jacobi(const cigpu_ham *base, int k, int l, double theta, cigpu_stream stream, cigpu_ham **out);

/* ---- DOCI pair scan: replaces LocalMinimizer::scan_orbitals (LocalMinimizer.cpp:73-128)
 * with DensDOCI::find_min_angle and calc_rotate (CIDens.cpp:1279-1464), on the device.
 * crs: a DOCI CRS (L <= 32); c: host, dim (its normalised ground state). For every
 * orbital pair k < l (index k*L + l - (k+1)(k+2)/2) the Newton search for the Jacobi
 * angle of lowest energy starts at 0.3 and, if it ends on a maximum, again at 0.01:
 * theta[p] is that angle, energy[p] the energy after the rotation (without Econst, as
 * calc_rotate returns it) and found[p] = 1 when it is a minimum with |theta| <= pi/2
 * (the pairs scan_orbitals keeps). Host outputs of L(L-1)/2 entries. ---- */
int cigpu_doci_pair_scan(cigpu_crs *crs, const double *c, double *theta, double *energy, int32_t *found);

/* ---- orbital optimisation: replaces OrbitalOptimization with its subclasses
 * SimulatedAnnealing (SimulatedAnnealing.cpp:42-156, 195-391) and LocalMinimizer
 * (LocalMinimizer.cpp:23-29, 73-280): the set_ham -> solve loop over rotated orbitals,
 * with every Hamiltonian, CRS, eigenvector and pair scan on the device. The
 * optimiser owns a device copy of the starting Hamiltonian (`ham` may be destroyed
 * after create), the current orbitals as a unitary U (row-major, U[a*L+p]: row a is
 * the current orbital a in the starting orbitals, as UnitaryMatrix stores it) with
 * their solved ground state, and the lowest energy seen with its unitary. ---- */
typedef struct cigpu_orbopt cigpu_orbopt;

typedef struct {
    int32_t method;      /* cigpu_method: the CIMethod whose energy is optimised */
    int32_t precision;   /* cigpu_precision of every build and solve */
    double tol;          /* FP64 residual target of every solve */
    int32_t warm_start;  /* 1: each solve starts from the current eigenvector (the
                            reference restarts ARPACK from scratch) */
    int32_t reserved;
    uint64_t seed;       /* random streams of the optimisers (splitmix64) */
} cigpu_orbopt_config;

/* SimulatedAnnealing(cim, temp, change_temp, angle, change_angle) and its loop
 * limits (SimulatedAnnealing.cpp:195-204, 306-391). */
typedef struct {
    double temp;           /* start temperature */
    double change_temp;    /* temperature factor per step */
    double max_angle;      /* start of the angle range: angle = max_angle (u1 - u2) */
    double change_angle;   /* angle-range factor per step */
    int64_t steps;         /* loop iterations (_c_steps, 20000 in the reference) */
    int64_t max_unaccept;  /* stop after more consecutive rejections (2000) */
    double min_angle;      /* stop when the angle range falls below (1e-7) */
    int32_t speculate;     /* at most this many proposals solved concurrently (1: one
                              at a time); the number follows the recent acceptance
                              rate (about 1 / rate); the chain is the same for every value */
    int32_t reserved;
} cigpu_anneal_params;

/* LocalMinimizer (LocalMinimizer.cpp:23-29, 130-235). */
typedef struct {
    double conv_crit;     /* |dE| counted as converged (1e-6) */
    int32_t conv_steps;   /* converged iterations to stop (25) */
    int32_t max_iters;    /* iteration limit (1000) */
    int32_t dist_choice;  /* 1: draw the pair by energy gain (choose_orbitalpair) */
    int32_t reserved;
} cigpu_local_params;

typedef struct {
    double e_current;       /* energy of the current orbitals, with Econst */
    double e_opt;           /* OrbitalOptimization::_opt_energy */
    int64_t solves;         /* builds + eigensolves */
    int64_t steps;          /* annealing steps decided / local iterations */
    int64_t accepted, rejected;
    int64_t speculative_waste;  /* solves of proposals discarded after an earlier acceptance */
    int64_t matvecs_fp64, matvecs_fp32;
    double seconds_rotate;  /* integral rotations, summed over solves (concurrent ones add up) */
    double seconds_build;   /* CRS builds, summed likewise */
    double seconds_solve;   /* eigensolves, summed likewise */
    double seconds_scan;    /* DOCI pair matrices + pair scan */
    double seconds;         /* wall time inside the optimiser calls */
} cigpu_orbopt_stats;

/* OrbitalOptimization(cim): copies the Hamiltonian and solves it (U = 1). */
int cigpu_orbopt_create(const cigpu_ham *ham, const cigpu_orbopt_config *cfg, cigpu_orbopt **out);
int cigpu_orbopt_destroy(cigpu_orbopt *opt);
/* SimulatedAnnealing::optimize; e_last = the energy of the final current orbitals
 * (the return value of the reference). Each call draws its proposals from a fresh
 * stream derived from the seed and the call count. */
int cigpu_orbopt_anneal(cigpu_orbopt *opt, const cigpu_anneal_params *p, double *e_last);
/* LocalMinimizer::optimize (DOCI only); e_final as returned by the reference.
 * CIGPU_ENOCONV when a scan finds no pair to rotate. */
int cigpu_orbopt_local(cigpu_orbopt *opt, const cigpu_local_params *p, double *e_final);
/* OrbitalOptimization::transform_orbitals + update_cim: one Jacobi rotation, solved. */
int cigpu_orbopt_jacobi(cigpu_orbopt *opt, int k, int l, double theta, double *e);
/* OrbitalOptimization::get_cim_no (density_method = the optimiser's method) or
 * get_fci_no (CIGPU_FCI): rotate to the natural orbitals of that method's ground
 * state in the current orbitals (SimulatedAnnealing.cpp:120-156) and solve. */
int cigpu_orbopt_natural(cigpu_orbopt *opt, int density_method, double *e);
/* OrbitalOptimization::set_cim_optimal: current orbitals = the best seen, solved. */
int cigpu_orbopt_set_optimal(cigpu_orbopt *opt);
/* Current state: U and U_opt (L*L), c (dim) and stats; each output optional. */
int cigpu_orbopt_get(const cigpu_orbopt *opt, double *U, double *U_opt, double *c, cigpu_orbopt_stats *stats);
/* A new Hamiltonian handle with the current orbitals' integrals (get_ham of the CIMethod). */
int cigpu_orbopt_ham(const cigpu_orbopt *opt, cigpu_ham **out);

#ifdef __cplusplus
}
#endif
#endif /* CIGPU_H */
