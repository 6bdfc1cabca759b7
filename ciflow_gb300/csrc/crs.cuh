// The CRS handle shared by the ABI, RDM and server translation units.
#pragma once

#include <memory>

#include "build.cuh"
#include "doci_mv.cuh"
#include "lanczos.cuh"
#include "sigma.cuh"
#include "slots.cuh"

namespace cigpu {
struct FciRdmPlan;  // rdm.cu
}

struct cigpu_crs {
    cigpu_ham *ham = nullptr;
    int method = CIGPU_FCI, precision = CIGPU_FP64;
    int L = 0, nup = 0, ndown = 0;
    int64_t dim = 0, nnz_full = 0, nnz_upper = 0;
    int device = -1;  // CUDA device the matrix lives on
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // FCI string tables (host copies kept for the RDM code)
    cigpu::SpinTables ta, tb;
    cigpu::SpinDevStore da, db;
    // DOCI pair strings
    cigpu::DevBuf<uint64_t> strings;
    // matrix
    cigpu::DevBuf<double> diag;
    cigpu::DevBuf<int64_t> row_ptr;
    cigpu::DevBuf<uint32_t> col, upper_off;
    cigpu::DevBuf<double> val64;
    cigpu::DevBuf<float> val32;
    cigpu::DevBuf<float> val32lo;  // MIXED: FP32 rounding remainder of each value
    // MIXED FCI: values-only slot tiles (val32/val32lo hold slots_count(fp) values,
    // no col); row_ptr/upper_off/nnz still describe the explicit matrix for export
    bool slots = false;
    // compact layouts allowed: FP64 slot tiles for FP64 FCI, the matrix-free pair-hop
    // form for DOCI (the lockstep batch concatenates explicit CRS matrices)
    bool allow_compact = true;
    // MIXED FCI: take the sigma FP32 product on any grid (builds whose solves run
    // beside others, as in the server and the batch, where GPU work per product
    // counts rather than one solve's latency)
    bool sigma_any_grid = false;
    // DOCI without a stored matrix: the matvecs generate the pair hops (doci_mv.cu)
    // from the strings and K_jk; row_ptr / upper_off are filled on demand (export)
    bool pairs = false;
    bool rows_ready = true;
    cigpu::DevBuf<double> kpair64;
    cigpu::DevBuf<float> kpair32, diag32;
    cigpu::DevBuf<uint64_t> slot_desc;  // the slot matvecs' staging tables (slot_tables_launch)
    cigpu::DevBuf<uint32_t> slot_st;
    cigpu::DevBuf<float> x32;  // MIXED: FP32 copy of x for the FP64 product from hi + lo
    // MIXED FCI: the FP32 product as a factorised direct-CI sigma vector (sigma.cu);
    // null when the space or the rank does not qualify (the FP32 slot values serve)
    std::unique_ptr<cigpu::SigmaOp> sig;
    cigpu::FciParams fp{};
    cigpu::DociParams dp{};
    // determinant lists (FCI_File / CI_Big)
    int det_words = 0;              // 64-bit words per spin string: 1 (L <= 64) or 2 (L <= 128)
    bool onthefly = false;          // CI_Big: elements recomputed in every matvec, outside a stored leading block
    int64_t det_block = 0;          // CI_Big: leading determinants whose block is stored (row_ptr / col / val64)
    cigpu::DevBuf<uint64_t> dets;   // [dim][2 * det_words]: up words, then down words
    double build_seconds = 0;
    std::shared_ptr<cigpu::FciRdmPlan> rdm_plan;  // FCI RDM plan, made by the first RDM call
    // A sigma-backed mixed FCI build leaves its FP64 fill, the slot staging tables
    // and the row counts running on `side`: the first Davidson cycle needs only the
    // string tables and the sigma factors. The FP64 products wait for side_done on
    // the device; the row counts are read, and the passes' temporaries released, by
    // the first call that needs them (finish_deferred).
    cudaStream_t side = nullptr;
    cudaEvent_t side_done = nullptr;
    bool counts_pending = false;
    std::shared_ptr<void> side_keep;

    ~cigpu_crs() {
        if (side) {
            cudaStreamSynchronize(side);
            side_keep.reset();
            cudaStreamDestroy(side);
        }
        if (side_done) cudaEventDestroy(side_done);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

namespace cigpu {
// cigpu_build with a choice of layout: fp64_tiles = false keeps an FP64 FCI matrix
// as a CRS (the lockstep batch concatenates CRS matrices).
int build_handle(cigpu_ham *ham, int method, int precision, cigpu_stream stream, bool fp64_tiles, cigpu_crs **out,
                 bool sigma_any_grid = false);
// Builds the CRS for `ham` on stream `s` (throws on failure).
void build_crs(cigpu_crs &c, cudaStream_t s);
// Waits for a deferred build pass and reads its row counts (no-op otherwise).
void finish_deferred(cigpu_crs &c);
// FP64 product y = H x on the CRS stream (device pointers).
void crs_mv64(cigpu_crs &c, const double *x, double *y, cudaStream_t s);
// FP32 product (MIXED CRS only).
void crs_mv32(cigpu_crs &c, const float *x, float *y, cudaStream_t s);
// Device bytes a build + solve of this shape needs.
size_t estimate_bytes(int L, int nup, int ndown, int method, int precision);
// RDMs of device vector c (normalised); host outputs as in cigpu_rdm.
void crs_rdm(cigpu_crs &c, const double *c_dev, double *rdm1, double *aa, double *ab, double *bb, cudaStream_t s);
int status_from_exception();
// y = H x of a determinant list without a stored matrix (every pair rescanned).
void dets_mv64(cigpu_crs &c, const double *x, double *y, cudaStream_t s);
// RDMs of a determinant list's state (device vector c); host outputs as cigpu_rdm
// (the 2-RDM when aa, ab and bb are all given).
void dets_rdm(cigpu_crs &c, const double *c_dev, double *rdm1, double *aa, double *ab, double *bb, cudaStream_t s);
// CIGPU_EINVAL unless h is symmetric and eri 8-fold symmetric (1e-10 relative) and all finite.
int validate_integrals(int L, const double *h, const double *eri, bool *exact);
// CIGPU_EINVAL unless U (L x L, row-major) is finite and orthogonal to 1e-10.
int validate_rotation(int L, const double *U);
// Lowest eigenpair of a built CRS with a device vector: c_dev holds the start when
// have_start, and the normalised eigenvector on return. Runs on `stream` (NULL:
// the CRS stream); info.e0 includes Econst. Returns CIGPU_OK or CIGPU_ENOCONV.
int solve_crs(cigpu_crs &crs, double tol, int64_t max_matvec, double *c_dev, bool have_start, cigpu_solve_info &info,
              cudaStream_t stream = nullptr);
// Rotated Hamiltonian h' = U h U^T, (ab|cd)' = sum U U U U (pq|rs) (host U, row-major).
void rotate_ham(const cigpu_ham &base, const double *U, cigpu_ham &H, cudaStream_t s);
// exp(X) of an antisymmetric L x L generator (host).
void unitary_exp(int L, const double *X, double *U);
// DOCI: blocks of partial sums doci_pair_matrices needs (partial holds 2 L^2 doubles per block).
int doci_pair_partials();
// DOCI pair matrices of device vector c (normalised): Pm[j][k] = Gamma_ab(jj,kk),
// Dm[j][k] = Gamma_aa(jk,jk) (zero diagonal); device outputs, L x L each.
void doci_pair_matrices(cigpu_crs &c, const double *c_dev, double *partial, double *Pm, double *Dm, cudaStream_t s);
}  // namespace cigpu

#define CIGPU_TRY try {
#define CIGPU_CATCH \
    }               \
    catch (...) { return status_from_exception(); }
