// C ABI of the cigpu library (include/cigpu.h): handles, build orchestration,
// export, matvec and solve entry points.
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "checked.cuh"
#include "crs.cuh"
#include "spmv.cuh"

namespace cigpu {

std::atomic<int64_t> g_launches{0};

// ---- caching device allocator ----
// Blocks are rounded up to 2 MiB (small requests to a power of two of at least
// 256 bytes) and kept per rounded size after release. A released block carries
// an event recorded on the releasing thread's stream (StreamScope); it is handed
// out again at once on that same stream, and to any other stream only once the
// event has completed, so concurrent solves on different streams never share a
// block that pending work still touches. A failed cudaMalloc returns every cached
// block to the driver and retries once.
namespace {
struct Cached {
    void *p;
    cudaEvent_t ev;   // completes when the releasing stream's work on the block is done
    cudaStream_t st;  // the releasing stream
};
std::mutex g_alloc_mutex;
std::multimap<size_t, Cached> g_free_blocks;  // rounded size -> block (current device)
std::map<void *, size_t> g_block_size;        // every live or cached block -> rounded size
std::vector<cudaEvent_t> g_event_pool;
size_t g_cached_bytes = 0, g_live_bytes = 0;
constexpr size_t kMaxCachedBytes = size_t(96) << 30;
thread_local cudaStream_t tls_stream = nullptr;
thread_local bool tls_stream_set = false;

size_t round_block(size_t bytes) {
    if (bytes >= (size_t(2) << 20)) return (bytes + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
    size_t r = 256;
    while (r < bytes) r <<= 1;
    return r;
}

void recycle_event_locked(cudaEvent_t ev) {
    if (ev) g_event_pool.push_back(ev);
}

bool reusable(const Cached &c) {
    if (!c.ev) return true;
    if (tls_stream_set && c.st == tls_stream) return true;  // stream order covers it
    const cudaError_t q = cudaEventQuery(c.ev);
    if (q == cudaSuccess) return true;
    if (cudaPeekAtLastError() == q) cudaGetLastError();  // "not ready" is not an error here
    return false;
}

void release_cache_locked() {
    for (auto &kv : g_free_blocks) {
        cudaFree(kv.second.p);  // synchronises the device: pending users are done
        g_block_size.erase(kv.second.p);
        recycle_event_locked(kv.second.ev);
    }
    g_free_blocks.clear();
    g_cached_bytes = 0;
}
}  // namespace

StreamScope::StreamScope(cudaStream_t s, bool set) : prev(tls_stream), prev_set(tls_stream_set) {
    tls_stream = s;
    tls_stream_set = set;
}

StreamScope::~StreamScope() {
    tls_stream = prev;
    tls_stream_set = prev_set;
}

void *dev_alloc(size_t bytes) {
    const size_t rb = round_block(bytes);
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    // best fit among cached blocks, wasting at most a quarter
    for (auto it = g_free_blocks.lower_bound(rb); it != g_free_blocks.end() && it->first <= rb + rb / 4; ++it) {
        if (!reusable(it->second)) continue;
        void *p = it->second.p;
        const size_t got = it->first;
        recycle_event_locked(it->second.ev);
        g_free_blocks.erase(it);
        g_cached_bytes -= got;
        g_live_bytes += got;
        return p;
    }
    void *p = nullptr;
    if (cudaMalloc(&p, rb) != cudaSuccess) {
        cudaGetLastError();
        release_cache_locked();
        if (cudaMalloc(&p, rb) != cudaSuccess) {
            cudaGetLastError();  // clear the allocation error
            throw std::bad_alloc();
        }
    }
    g_block_size[p] = rb;
    g_live_bytes += rb;
    return p;
}

void dev_free(void *p, size_t) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    auto it = g_block_size.find(p);
    if (it == g_block_size.end()) return;
    const size_t rb = it->second;
    g_live_bytes -= rb;
    if (g_cached_bytes + rb > kMaxCachedBytes) {
        cudaFree(p);
        g_block_size.erase(it);
        return;
    }
    Cached c{p, nullptr, nullptr};
    if (tls_stream_set) {
        if (!g_event_pool.empty()) {
            c.ev = g_event_pool.back();
            g_event_pool.pop_back();
        } else if (cudaEventCreateWithFlags(&c.ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            c.ev = nullptr;
        }
        if (c.ev && cudaEventRecord(c.ev, tls_stream) != cudaSuccess) {
            cudaGetLastError();
            recycle_event_locked(c.ev);
            c.ev = nullptr;
        }
        c.st = tls_stream;
        if (!c.ev) cudaStreamSynchronize(tls_stream);
    } else {
        cudaDeviceSynchronize();  // unknown stream: wait as cudaFree would
    }
    g_free_blocks.emplace(rb, c);
    g_cached_bytes += rb;
}

size_t dev_bytes_in_use() {
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    return g_live_bytes;
}

void SpinDevStore::upload(const SpinTables &t, cudaStream_t s) {
    auto up = [&](auto &buf, const auto &vec) {
        using T = typename std::decay_t<decltype(vec)>::value_type;
        buf.alloc(vec.size());
        if (!vec.empty())
            CIGPU_CUDA(cudaMemcpyAsync(buf.p, vec.data(), vec.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    };
    up(occ, t.occ);
    up(diag, t.diag);
    up(s_target, t.s_target);
    up(s_part, t.s_part);
    up(s_info, t.s_info);
    up(d_target, t.d_target);
    up(d_val, t.d_val);
    up(d_hi, t.d_hi);
    up(d_lo, t.d_lo);
    up(nb_full, t.nb_full);
    up(nb_sing, t.nb_sing);
    view = SpinDev{t.D, t.n, t.ns, t.nd, t.nfull, t.nsing, occ.p, diag.p, s_target.p, s_part.p,
                   s_info.p, d_target.p, d_val.p, d_hi.p, d_lo.p, nb_full.p, nb_sing.p};
}

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Every Trace is also an NVTX range ("cigpu <scope>") with a marker at each phase
// end, so a profiler timeline shows the phases without CIGPU_TRACE.
Trace::Trace(const char *sc, cudaStream_t st) : scope(sc), s(st) {
    const char *e = std::getenv("CIGPU_TRACE");
    on = e && e[0] == '1';
    t0 = now_s();
    char name[64];
    std::snprintf(name, sizeof(name), "cigpu %s", sc);
    nvtxRangePushA(name);
}

Trace::~Trace() { nvtxRangePop(); }

void Trace::mark(const char *what) {
    nvtxMarkA(what);
    if (!on) return;
    cudaStreamSynchronize(s);
    const double t = now_s();
    std::fprintf(stderr, "[cigpu %s] %-24s %9.3f ms\n", scope, what, (t - t0) * 1e3);
    t0 = t;
}

// The checked build's error word, one per device, allocated and cleared on first use.
unsigned long long *check_word_device() {
#if CIGPU_CHECKED_BUILD
    constexpr int kMaxDev = 64;
    static std::mutex mu;
    static unsigned long long *words[kMaxDev] = {nullptr};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!words[dev]) {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(unsigned long long)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(unsigned long long)) != cudaSuccess) return nullptr;
        words[dev] = static_cast<unsigned long long *>(p);
    }
    return words[dev];
#else
    return nullptr;
#endif
}

int status_from_exception() {
    try {
        throw;
    } catch (const CudaError &e) {
        std::fprintf(stderr, "cigpu: CUDA error %s in %s\n", cudaGetErrorString(e.err), e.what);
        return CIGPU_ECUDA;
    } catch (const std::bad_alloc &) {
        return CIGPU_ENOMEM;
    } catch (const std::invalid_argument &) {
        return CIGPU_EINVAL;
    } catch (...) {
        return CIGPU_ECUDA;
    }
}

static int64_t binom64(int n, int k) { return d_binom(n, k); }

// The mixed FCI method's FP32 product, read at every build from CIGPU_FP32_PRODUCT:
// "slots" takes the stored FP32 slot values, "sigma" the factorised sigma operator
// on any space it supports, anything else the sigma operator where its tile grid
// fills the GPU. Both are complete products; the choice exists to compare them.
enum SigmaMode { kSigmaOff = 0, kSigmaAuto = 1, kSigmaForced = 2 };
int sigma_mode() {
    const char *e = std::getenv("CIGPU_FP32_PRODUCT");
    if (e && std::strcmp(e, "slots") == 0) return kSigmaOff;
    if (e && std::strcmp(e, "sigma") == 0) return kSigmaForced;
    return kSigmaAuto;
}

// FP64 slot tiles, read at every build from CIGPU_SLOTS64: "compact" leaves out the
// alpha-single x beta-single block (the matvec forms it from the integrals) wherever
// its tables fit, anything else stores every slot. The products are the same bit
// for bit. Compact tiles hold 3.4x fewer values at L=12 6a6b (3.8 against 13.0 GB)
// and fill faster (whole build 5.5 against 8.3 ms), but their product takes 3.8
// against 2.7 ms: forming the block is bound by the shared-memory and L1 gathers
// (its integrals and x), not by the FP64 pipe. A mixed solve's three FP64 anchors
// then cost more than the smaller fill saves (55.1 against 54.1 ms per build +
// solve), so the full tiles are the default and the compact ones a memory saver.
bool slots64_compact() {
    const char *e = std::getenv("CIGPU_SLOTS64");
    return e && std::strcmp(e, "compact") == 0;
}

size_t estimate_bytes(int L, int nup, int ndown, int method, int precision) {
    int64_t dim, W;
    dim = std::max<int64_t>(space_dim(method, L, nup, ndown), 0);
    if (method == CIGPU_DOCI) {
        W = 1 + (int64_t)nup * (L - nup);
    } else {
        const int64_t sa = (int64_t)nup * (L - nup), sb = (int64_t)ndown * (L - ndown);
        W = 1 + sa + sb + sa * sb + binom64(nup, 2) * binom64(L - nup, 2) + binom64(ndown, 2) * binom64(L - ndown, 2);
    }
    const size_t vbytes = precision == CIGPU_MIXED ? 4 : 8;
    // col + values (FP64, or FP32 hi + lo); the mixed FCI layout stores values only
    size_t b = (size_t)dim * W * 12;
    if (method == CIGPU_FCI && precision == CIGPU_MIXED) {  // slot tiles of kTileRows beta strings, hi + lo
        b = (size_t)binom64(L, nup) * ((binom64(L, ndown) + kTileRows - 1) / kTileRows * kTileRows) * (W + 16) * 8;
        if (sigma_applies(L))  // the FP32 sigma operator at its largest rank
            b += sigma_bytes(L, binom64(L, nup), binom64(L, ndown),
                             std::min(kSigmaMaxRank, (L * (L + 1) / 2 + kSigmaChunk - 1) / kSigmaChunk * kSigmaChunk));
    }
    if (method == CIGPU_DOCI)  // matrix-free: strings and the FP32 diagonal
        b = (size_t)dim * (8 + 4);
    b += (size_t)dim * (8 + 8 + 4 + 4);          // row_ptr, diag, counts, upper offsets
    b += (size_t)dim * vbytes * (42 + 1 + 14);   // Krylov basis + restart buffer
    b += (size_t)dim * 8 * 5;                    // c, refinement vectors
    b += (size_t)L * L * L * L * 8 + (64u << 20);  // integrals + tables/slack
    return b;
}

// Per-row single-excitation tables of an FCI CRS (FP64, plus the FP32 splits of
// them and of the diagonal for MIXED); only the fill passes read them.
struct RowSingles {
    DevBuf<double> sgl64;
    DevBuf<float> sgl_hi, sgl_lo, diag_hi, diag_lo;
    // fp32: also the FP32 splits (the FP32 fills read them)
    void make(cigpu_crs &c, FciParams &p, cudaStream_t s, bool fp32) {
        const size_t nsr = (size_t)(c.da.view.ns + c.db.view.ns);
        sgl64.alloc(std::max<size_t>((size_t)c.dim * nsr, 1));
        if (fp32) {
            sgl_hi.alloc(std::max<size_t>((size_t)c.dim * nsr, 1));
            sgl_lo.alloc(std::max<size_t>((size_t)c.dim * nsr, 1));
            diag_hi.alloc(c.dim);
            diag_lo.alloc(c.dim);
        }
        fci_singles_launch(p, sgl64.p, sgl_hi.p, sgl_lo.p, diag_hi.p, diag_lo.p, s);
        p.sgl64 = sgl64.p;
        p.sgl_hi = sgl_hi.p;
        p.sgl_lo = sgl_lo.p;
        p.diag_hi = diag_hi.p;
        p.diag_lo = diag_lo.p;
    }
};

// Temporaries of the build passes, kept with the handle while a deferred pass runs.
struct BuildTemps {
    RowSingles singles;
    DevBuf<uint32_t> count;
    DevBuf<int64_t> urow, sums1, sums2;
};

void finish_deferred(cigpu_crs &c) {
    if (!c.counts_pending) return;
    CIGPU_CUDA(cudaEventSynchronize(c.side_done));
    auto *t = static_cast<BuildTemps *>(c.side_keep.get());
    CIGPU_CUDA(cudaMemcpy(&c.nnz_full, c.row_ptr.p + c.dim, sizeof(int64_t), cudaMemcpyDeviceToHost));
    CIGPU_CUDA(cudaMemcpy(&c.nnz_upper, t->urow.p + c.dim, sizeof(int64_t), cudaMemcpyDeviceToHost));
    c.side_keep.reset();
    c.counts_pending = false;
}

// Explicit FP32 CRS (columns + hi values) of a values-only CRS, for export.
// The explicit CRS (columns and values) of a matrix stored as slot tiles, made by
// the CRS generator for export: FP32 hi/lo values for MIXED, FP64 for FP64.
struct ExplicitCrs {
    DevBuf<uint32_t> col;
    DevBuf<float> hi, lo;
    DevBuf<double> v64;
    void make(cigpu_crs &c, cudaStream_t s) {
        if (c.pairs) {
            make_doci(c, s);
            return;
        }
        FciParams q = c.fp;
        RowSingles rs;
        rs.make(c, q, s, c.precision == CIGPU_MIXED);
        col.alloc(std::max<int64_t>(c.nnz_full, 1));
        q.row_ptr = c.row_ptr.p;
        q.col = col.p;
        if (c.precision == CIGPU_FP64) {
            v64.alloc(std::max<int64_t>(c.nnz_full, 1));
            q.val64 = v64.p;
            fci_launch(kFill64, q, s);
        } else {
            hi.alloc(std::max<int64_t>(c.nnz_full, 1));
            lo.alloc(std::max<int64_t>(c.nnz_full, 1));
            q.val32 = hi.p;
            q.val32lo = lo.p;
            fci_launch(kFill32, q, s);
        }
    }
    // DOCI without a stored matrix: the row structure (count pass + scan, kept in
    // the handle) and the explicit rows from the CRS generator.
    void make_doci(cigpu_crs &c, cudaStream_t s) {
        DociParams q = c.dp;
        if (!c.rows_ready) {
            DevBuf<uint32_t> count(c.dim);
            q.row_count = count.p;
            q.upper_off = c.upper_off.p;
            doci_launch(kCount, q, s);
            exclusive_scan_u32(count.p, c.row_ptr.p, c.dim, s);
            CIGPU_CUDA(cudaStreamSynchronize(s));
            c.rows_ready = true;
        }
        col.alloc(std::max<int64_t>(c.nnz_full, 1));
        q.row_ptr = c.row_ptr.p;
        q.col = col.p;
        if (c.precision == CIGPU_FP64) {
            v64.alloc(std::max<int64_t>(c.nnz_full, 1));
            q.val64 = v64.p;
            doci_launch(kFill64, q, s);
        } else {
            hi.alloc(std::max<int64_t>(c.nnz_full, 1));
            lo.alloc(std::max<int64_t>(c.nnz_full, 1));
            q.val32 = hi.p;
            q.val32lo = lo.p;
            doci_launch(kFill32, q, s);
        }
    }
};

void build_crs(cigpu_crs &c, cudaStream_t s) {
    const auto t0 = std::chrono::steady_clock::now();
    CIGPU_CUDA(cudaGetDevice(&c.device));
    Trace tr("build", s);
    cigpu_ham &h = *c.ham;
    const int64_t dim = c.dim;
    c.diag.alloc(dim);
    auto temps = std::make_shared<BuildTemps>();
    temps->count.alloc(dim);
    DevBuf<uint32_t> &count = temps->count;
    RowSingles &singles = temps->singles;  // FCI row singles (build only)
    cudaStream_t fs = s;                    // stream of the fill, staging tables and counts
    c.upper_off.alloc(dim);
    c.row_ptr.alloc(dim + 1);
    tr.mark("alloc small");
    if (c.method == CIGPU_FCI) {
        if (!h.host_valid) throw std::logic_error("FCI build needs the host copy of the integrals");
        build_spin_tables(c.L, c.nup, h.h.data(), h.eri.data(), c.ta);
        tr.mark("host tables");
        c.da.upload(c.ta, s);
        if (c.ndown == c.nup) {
            c.db.view = c.da.view;
        } else {
            build_spin_tables(c.L, c.ndown, h.h.data(), h.eri.data(), c.tb);
            c.db.upload(c.tb, s);
        }
        FciParams &p = c.fp;
        p.L = c.L;
        p.Db = c.db.view.D;
        p.a = c.da.view;
        p.b = c.db.view;
        p.eri = h.d_eri.p;
        p.eri_hi = h.d_eri_hi.p;
        p.eri_lo = h.d_eri_lo.p;
        p.diag = c.diag.p;
        fci_diag_launch(p, c.diag.p, s);
        c.slots = slots_supported(p) &&
                  (c.precision == CIGPU_MIXED || (c.allow_compact && slots64_pay(p)));
        // MIXED: the FP32 products as the factorised sigma vector where it applies
        // (its factorisation runs on the host while the diagonal is computed)
        const int smode = sigma_mode();
        if (c.slots && c.precision == CIGPU_MIXED && c.allow_compact && sigma_applies(c.L) && smode != kSigmaOff) {
            c.sig.reset(new SigmaOp);
            if (!sigma_prepare(*c.sig, c.L, h.h.data(), h.eri.data(), c.ta, c.ndown == c.nup ? c.ta : c.tb,
                               smode == kSigmaForced || c.sigma_any_grid, s))
                c.sig.reset();
            tr.mark("sigma factors");
        }
        if (c.sig) {
            // the rest runs beside the solve's first Davidson cycle (see cigpu_crs::side);
            // it starts after everything queued on s so far
            CIGPU_CUDA(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
            CIGPU_CUDA(cudaEventCreateWithFlags(&c.side_done, cudaEventDisableTiming));
            cudaEvent_t ready = nullptr;
            CIGPU_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
            CIGPU_CUDA(cudaEventRecord(ready, s));
            CIGPU_CUDA(cudaStreamWaitEvent(c.side, ready, 0));
            CIGPU_CUDA(cudaEventDestroy(ready));
            fs = c.side;
        }
        // FP32 splits only for a fill of FP32 values (not for the FP64 values of the
        // sigma-backed mixed form)
        singles.make(c, p, fs, c.precision == CIGPU_MIXED && !c.sig);
        tr.mark("upload + diag + singles");
        p.row_count = count.p;
        p.upper_off = c.upper_off.p;
        if (c.slots) {
            // values-only layout: the fill counts the rows itself; MIXED stores FP32
            // hi + lo for its FP32 and FP64 products, or, with the sigma vector doing
            // the FP32 ones, the FP64 values (its anchors take the plain FP64 product)
            if (c.precision == CIGPU_MIXED && !c.sig) {
                c.val32.alloc(slots_count(p));
                c.val32lo.alloc(slots_count(p));
                fill_slots_launch(p, c.val32.p, c.val32lo.p, count.p, c.upper_off.p, fs);
            } else {
                p.fly = slots64_compact() && slots64_fly_fits(p) ? 1 : 0;
                c.val64.alloc(std::max<int64_t>(slots_stored(p), 4));
                fill_slots64_launch(p, c.val64.p, count.p, c.upper_off.p, fs);
            }
            c.slot_desc.alloc(std::max<int64_t>(slot_desc_count(p), 1));
            c.slot_st.alloc(std::max<int64_t>(slot_st_count(p), 4));
            slot_tables_launch(p, c.slot_desc.p, c.slot_st.p, fs);
            p.desc_tab = c.slot_desc.p;
            p.st_tab = c.slot_st.p;
            tr.mark("slot fill");
        } else {
            fci_launch(kCount, p, s);
            tr.mark("count pass");
        }
    } else {
        c.strings.alloc(dim);
        doci_strings_launch(c.L, c.nup, dim, c.strings.p, s);
        DociParams &p = c.dp;
        p.L = c.L;
        p.n = c.nup;
        p.W = 1 + c.nup * (c.L - c.nup);
        p.D = dim;
        p.fullmask = c.L >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << c.L) - 1);
        p.strings = c.strings.p;
        p.h = h.d_h.p;
        p.eri = h.d_eri.p;
        p.diag = c.diag.p;
        doci_diag_launch(p, c.diag.p, s);
        p.row_count = count.p;
        p.upper_off = c.upper_off.p;
        // MIXED is matrix-free (its FP32 product costs about what the FP32 CRS costs,
        // and the build drops from a CRS count + sort + fill to the pair table); the
        // FP64 form keeps the CRS, whose FP64 product is the faster one (1.24 against
        // 1.70 ms at L=24, 12 pairs), and its 120-odd matvecs outweigh the build
        if (c.allow_compact && c.precision == CIGPU_MIXED) {
            // matrix-free: the pair-hop table and, for MIXED, the FP32 diagonal; the
            // stored-element counts follow from K: a pair (j, k) with K_jk != 0 hops in
            // the C(L-2, n-1) strings holding j and not k
            const int L = c.L, n = c.nup;
            c.pairs = true;
            c.rows_ready = false;
            c.kpair64.alloc((size_t)L * L);
            c.kpair32.alloc((size_t)L * L);
            doci_pair_table_launch(L, h.d_eri.p, c.kpair64.p, c.kpair32.p, s);
            if (c.precision == CIGPU_MIXED) {
                c.diag32.alloc(dim);
                dev_convert(c.diag.p, c.diag32.p, dim, s);
            }
            std::vector<double> K((size_t)L * L);
            CIGPU_CUDA(cudaMemcpyAsync(K.data(), c.kpair64.p, sizeof(double) * K.size(), cudaMemcpyDeviceToHost, s));
            const int64_t nd = count_nonzero(c.diag.p, dim, s);  // synchronises s
            int64_t nk = 0, nku = 0;
            for (int j = 0; j < L; ++j)
                for (int k = 0; k < L; ++k)
                    if (K[(size_t)j * L + k] != 0.0) {
                        ++nk;
                        nku += k > j;
                    }
            const int64_t per = (n >= 1 && L >= 2) ? d_binom(L - 2, n - 1) : 0;
            c.nnz_full = nd + nk * per;
            c.nnz_upper = nd + nku * per;
            tr.mark("strings + diag + pair table");
            c.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            return;
        }
        doci_launch(kCount, p, s);
        tr.mark("strings + diag + count");
    }
    if (c.side) {
        // deferred: the scans on the side stream, the counts read by finish_deferred
        exclusive_scan_u32_async(count.p, c.row_ptr.p, dim, temps->sums1, fs);
        temps->urow.alloc(dim + 1);
        upper_counts_launch(dim, c.row_ptr.p, c.upper_off.p, count.p, fs);
        exclusive_scan_u32_async(count.p, temps->urow.p, dim, temps->sums2, fs);
        CIGPU_CUDA(cudaEventRecord(c.side_done, fs));
        c.side_keep = temps;
        c.counts_pending = true;
        tr.mark("deferred passes queued");
        CIGPU_CUDA(cudaStreamSynchronize(s));
        c.fp.sgl64 = nullptr;
        c.fp.sgl_hi = c.fp.sgl_lo = c.fp.diag_hi = c.fp.diag_lo = nullptr;
        c.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return;
    }
    exclusive_scan_u32(count.p, c.row_ptr.p, dim, s);
    CIGPU_CUDA(cudaMemcpyAsync(&c.nnz_full, c.row_ptr.p + dim, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    // upper-triangle size (the reference CRS)
    {
        upper_counts_launch(dim, c.row_ptr.p, c.upper_off.p, count.p, s);
        DevBuf<int64_t> urow(dim + 1);
        exclusive_scan_u32(count.p, urow.p, dim, s);
        CIGPU_CUDA(cudaMemcpyAsync(&c.nnz_upper, urow.p + dim, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaStreamSynchronize(s));
    }
    count.release();
    tr.mark("scans");
    const int mode = c.precision == CIGPU_MIXED ? kFill32 : kFill64;
    if (c.slots) {
        // filled above
    } else if (mode == kFill64) {
        c.col.alloc(c.nnz_full);
        c.val64.alloc(c.nnz_full);
    } else {
        c.col.alloc(c.nnz_full);
        c.val32.alloc(c.nnz_full);
        c.val32lo.alloc(c.nnz_full);
    }
    tr.mark("alloc matrix");
    if (c.method == CIGPU_FCI) {
        c.fp.row_ptr = c.row_ptr.p;
        c.fp.col = c.col.p;
        c.fp.val64 = c.val64.p;
        c.fp.val32 = c.val32.p;
        c.fp.val32lo = c.val32lo.p;
        if (!c.slots) fci_launch(mode, c.fp, s);
    } else {
        c.dp.row_ptr = c.row_ptr.p;
        c.dp.col = c.col.p;
        c.dp.val64 = c.val64.p;
        c.dp.val32 = c.val32.p;
        c.dp.val32lo = c.val32lo.p;
        doci_launch(mode, c.dp, s);
    }
    tr.mark("fill pass");
    CIGPU_CUDA(cudaStreamSynchronize(s));
    // the per-row singles tables are only needed by the build passes
    c.fp.sgl64 = nullptr;
    c.fp.sgl_hi = c.fp.sgl_lo = c.fp.diag_hi = c.fp.diag_lo = nullptr;
    c.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void crs_mv64(cigpu_crs &c, const double *x, double *y, cudaStream_t s) {
    if (c.onthefly) {
        dets_mv64(c, x, y, s);
        return;
    }
    if (c.pairs) {
        doci_mv64(DociMv{c.L, c.nup, c.dim, c.strings.p}, c.kpair64.p, c.diag.p, x, y, s);
        return;
    }
    if (c.slots && c.val64.p) {  // FP64 slot values: the plain method, or MIXED with the sigma vector
        if (c.side_done) CIGPU_CUDA(cudaStreamWaitEvent(s, c.side_done, 0));  // a deferred fill
        spmv_slots_f64(c.fp, c.val64.p, x, y, s);
        return;
    }
    if (c.precision == CIGPU_MIXED) {
        if (!c.x32.p) c.x32.alloc(std::max<int64_t>(c.dim, 1));
        dev_convert(x, c.x32.p, c.dim, s);
    }
    if (c.slots) {
        spmv_slots_hilo(c.fp, c.val32.p, c.val32lo.p, x, c.x32.p, y, s);
        return;
    }
    if (c.precision == CIGPU_FP64) {
        spmv_f64(c.dim, c.nnz_full, c.row_ptr.p, c.col.p, c.val64.p, x, y, s);
        return;
    }
    if (c.val32lo.p || c.nnz_full == 0) {
        // MIXED CRS: FP64 product with values hi + lo (|v - hi - lo| <= 2^-48 |v|);
        // an all-zero matrix (e.g. no electrons) has no value arrays at all
        spmv_hilo(c.dim, c.nnz_full, c.row_ptr.p, c.col.p, c.val32.p, c.val32lo.p, x, c.x32.p, y, s);
        return;
    }
    throw std::invalid_argument("MIXED CRS without its FP32 remainder array");
}

void crs_mv32(cigpu_crs &c, const float *x, float *y, cudaStream_t s) {
    if (c.precision != CIGPU_MIXED || c.onthefly) throw std::invalid_argument("FP32 matvec needs a MIXED CRS");
    if (c.pairs) {
        doci_mv32(DociMv{c.L, c.nup, c.dim, c.strings.p}, c.kpair32.p, c.diag32.p, x, y, s);
        return;
    }
    if (c.sig) {
        sigma_mv32(*c.sig, c.fp, x, y, s);
        return;
    }
    if (c.slots) {
        spmv_slots_f32(c.fp, c.val32.p, x, y, s);
        return;
    }
    spmv_f32(c.dim, c.nnz_full, c.row_ptr.p, c.col.p, c.val32.p, x, y, s);
}

// Host validation of integrals: finite, h symmetric, eri 8-fold symmetric to 1e-10
// relative. *exact reports whether eri is exactly symmetric already.
int validate_integrals(int L, const double *h, const double *eri, bool *exact_out) {
    const size_t L1 = L, L2 = L1 * L1, L3 = L2 * L1, L4 = L3 * L1;
    double hmax = 0, emax = 0;
    for (size_t i = 0; i < L2; ++i) {
        if (!std::isfinite(h[i])) return CIGPU_EINVAL;
        hmax = std::max(hmax, std::fabs(h[i]));
    }
    for (size_t i = 0; i < L4; ++i) {
        if (!std::isfinite(eri[i])) return CIGPU_EINVAL;
        emax = std::max(emax, std::fabs(eri[i]));
    }
    const double htol = 1e-10 * std::max(1.0, hmax), etol = 1e-10 * std::max(1.0, emax);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j)
            if (std::fabs(h[i * L1 + j] - h[j * L1 + i]) > htol) return CIGPU_EINVAL;
    bool exact = true;
    for (int p = 0; p < L; ++p)
        for (int q = 0; q < L; ++q)
            for (int r = 0; r < L; ++r)
                for (int s = 0; s < L; ++s) {
                    const double v = eri[p * L3 + q * L2 + r * L1 + s];
                    const double a = eri[q * L3 + p * L2 + r * L1 + s];
                    const double b = eri[r * L3 + s * L2 + p * L1 + q];
                    const double c = eri[p * L3 + q * L2 + s * L1 + r];
                    if (std::fabs(v - a) > etol || std::fabs(v - b) > etol || std::fabs(v - c) > etol)
                        return CIGPU_EINVAL;
                    exact = exact && v == a && v == b && v == c;
                }
    if (exact_out) *exact_out = exact;
    return CIGPU_OK;
}

int solve_crs(cigpu_crs &crs, double tol, int64_t max_matvec, double *c_dev, bool have_start, cigpu_solve_info &info,
              cudaStream_t stream) {
    cudaStream_t s = stream ? stream : crs.stream;
    Trace tr("solve", s);  // an NVTX range around the eigensolve
    cigpu_crs *cp = &crs;
    SolveProblem P;
    P.n = crs.dim;
    P.stream = s;
    P.diag = crs.diag.p;
    P.mv64 = [cp](const double *x, double *y, cudaStream_t st) { crs_mv64(*cp, x, y, st); };
    if (crs.precision == CIGPU_MIXED)
        P.mv32 = [cp](const float *x, float *y, cudaStream_t st) { crs_mv32(*cp, x, y, st); };
    P.fp32_first_anchor = crs.sig != nullptr;
    SolveOptions o;
    o.tol = tol;
    o.max_matvec = max_matvec;
    info = cigpu_solve_info{};
    const int st = crs.precision == CIGPU_MIXED ? solve_mixed(P, o, c_dev, have_start, info)
                                                : solve_fp64(P, o, c_dev, have_start, info);
    info.e0 += crs.ham->econst;
    info.precision = crs.precision;
    // a deferred build part that has completed by now: read its counts and release
    // its temporaries (the FP64 row singles among them) without waiting
    if (crs.counts_pending) {
        const cudaError_t q = cudaEventQuery(crs.side_done);
        if (q == cudaSuccess)
            finish_deferred(crs);
        else if (cudaPeekAtLastError() == q)
            cudaGetLastError();  // "not ready" is not an error here
    }
    return st;
}

}  // namespace cigpu

using namespace cigpu;

extern "C" {

int cigpu_get_version(void) { return CIGPU_ABI_VERSION; }

int cigpu_checked_build(void) { return CIGPU_CHECKED_BUILD; }

int cigpu_check_word(uint64_t *word, int reset) {
    if (!word) return CIGPU_EINVAL;
    *word = 0;
    if (!CIGPU_CHECKED_BUILD) return CIGPU_ENOTSUP;
    unsigned long long *w = check_word_device();
    if (!w) return CIGPU_ECUDA;
    unsigned long long h = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return CIGPU_ECUDA;
    if (cudaMemcpy(&h, w, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return CIGPU_ECUDA;
    if (reset && cudaMemset(w, 0, sizeof(*w)) != cudaSuccess) return CIGPU_ECUDA;
    *word = h;
    return CIGPU_OK;
}

const char *cigpu_strerror(int st) {
    switch (st) {
        case CIGPU_OK: return "ok";
        case CIGPU_EINVAL: return "invalid argument";
        case CIGPU_ENOMEM: return "out of memory or over the HBM budget";
        case CIGPU_EAGAIN: return "queue full, retry";
        case CIGPU_ECANCELED: return "cancelled";
        case CIGPU_ETIMEDOUT: return "timed out";
        case CIGPU_ENOTSUP: return "not supported";
        case CIGPU_ENOCONV: return "eigensolver did not converge";
        case CIGPU_ECUDA: return "CUDA error or no usable GPU";
        case CIGPU_ENOTFOUND: return "unknown request";
        default: return "unknown status";
    }
}

int cigpu_device_count(int *count) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    if (count) *count = n;
    return n > 0 ? CIGPU_OK : CIGPU_ECUDA;
}

int64_t cigpu_kernel_launches(void) { return g_launches.load(); }

int cigpu_ham_create(int L, int nup, int ndown, double econst, const double *h, const double *eri, cigpu_ham **out) {
    if (!out || !h || !eri) return CIGPU_EINVAL;
    *out = nullptr;
    if (L < 1 || L > kMaxLDets || nup < 0 || ndown < 0 || nup > L || ndown > L) return CIGPU_EINVAL;
    if (!std::isfinite(econst)) return CIGPU_EINVAL;
    const size_t L1 = L, L2 = L1 * L1, L3 = L2 * L1, L4 = L3 * L1;
    bool exact = true;
    if (validate_integrals(L, h, eri, &exact) != CIGPU_OK) return CIGPU_EINVAL;
    CIGPU_TRY
    StreamScope scope(nullptr, false);  // synchronous copies below: reuse only completed blocks
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return CIGPU_ECUDA;
    }
    std::unique_ptr<cigpu_ham> H(new cigpu_ham);
    H->L = L;
    H->nup = nup;
    H->ndown = ndown;
    H->econst = econst;
    H->h.assign(h, h + L2);
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < i; ++j) H->h[i * L1 + j] = H->h[j * L1 + i];
    H->eri.assign(eri, eri + L4);
    if (!exact) {
        // tolerate round-off asymmetry: every permutation takes the value of its
        // canonical representative (p>=q, r>=s, pq>=rs)
        for (int p = 0; p < L; ++p)
            for (int q = 0; q < L; ++q)
                for (int r = 0; r < L; ++r)
                    for (int s = 0; s < L; ++s) {
                        int a = std::max(p, q), b = std::min(p, q), c = std::max(r, s), d = std::min(r, s);
                        if (a * L + b < c * L + d) {
                            std::swap(a, c);
                            std::swap(b, d);
                        }
                        H->eri[p * L3 + q * L2 + r * L1 + s] = eri[a * L3 + b * L2 + c * L1 + d];
                    }
    }
    H->d_h.alloc(L2);
    H->d_eri.alloc(L4);
    CIGPU_CUDA(cudaMemcpy(H->d_h.p, H->h.data(), L2 * sizeof(double), cudaMemcpyHostToDevice));
    CIGPU_CUDA(cudaMemcpy(H->d_eri.p, H->eri.data(), L4 * sizeof(double), cudaMemcpyHostToDevice));
    {
        std::vector<float> hi(L4), lo(L4);
        for (size_t i = 0; i < L4; ++i) split_fp32(H->eri[i], hi[i], lo[i]);
        H->d_eri_hi.alloc(L4);
        H->d_eri_lo.alloc(L4);
        CIGPU_CUDA(cudaMemcpy(H->d_eri_hi.p, hi.data(), L4 * sizeof(float), cudaMemcpyHostToDevice));
        CIGPU_CUDA(cudaMemcpy(H->d_eri_lo.p, lo.data(), L4 * sizeof(float), cudaMemcpyHostToDevice));
    }
    *out = H.release();
    return CIGPU_OK;
    CIGPU_CATCH
}

int cigpu_ham_destroy(cigpu_ham *ham) {
    delete ham;
    return CIGPU_OK;
}

int cigpu_estimate_bytes(int L, int nup, int ndown, int method, int precision, size_t *bytes) {
    if (!bytes || L < 1 || L > kMaxL || nup < 0 || ndown < 0 || nup > L || ndown > L) return CIGPU_EINVAL;
    if (method != CIGPU_FCI && method != CIGPU_DOCI) return CIGPU_EINVAL;
    *bytes = estimate_bytes(L, nup, ndown, method, precision);
    return CIGPU_OK;
}

int cigpu_build(cigpu_ham *ham, int method, int precision, cigpu_stream stream, cigpu_crs **out) {
    return build_handle(ham, method, precision, stream, true, out);
}

}  // extern "C"

namespace cigpu {
int build_handle(cigpu_ham *ham, int method, int precision, cigpu_stream stream, bool compact, cigpu_crs **out,
                 bool sigma_any_grid) {
    if (!ham || !out) return CIGPU_EINVAL;
    *out = nullptr;
    if (method != CIGPU_FCI && method != CIGPU_DOCI) return CIGPU_EINVAL;
    if (precision != CIGPU_FP64 && precision != CIGPU_MIXED) return CIGPU_EINVAL;
    if (method == CIGPU_DOCI && ham->nup != ham->ndown) return CIGPU_EINVAL;
    if (method == CIGPU_DOCI && ham->nup > 32) return CIGPU_ENOTSUP;
    if (ham->L > kMaxL) return CIGPU_ENOTSUP;  // 64-bit strings; determinant lists go up to 128 orbitals
    const int64_t dim = space_dim(method, ham->L, ham->nup, ham->ndown);
    if (dim < 1 || dim > (int64_t)UINT32_MAX) return CIGPU_ENOTSUP;
    CIGPU_TRY
    std::unique_ptr<cigpu_crs> c(new cigpu_crs);
    c->ham = ham;
    c->method = method;
    c->precision = precision;
    c->L = ham->L;
    c->nup = ham->nup;
    c->ndown = ham->ndown;
    c->dim = dim;
    c->allow_compact = compact;
    c->sigma_any_grid = sigma_any_grid;
    if (stream) {
        c->stream = static_cast<cudaStream_t>(stream);
    } else {
        CIGPU_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    StreamScope scope(c->stream);
    build_crs(*c, c->stream);
    *out = c.release();
    return CIGPU_OK;
    CIGPU_CATCH
}
}  // namespace cigpu

extern "C" {

int cigpu_crs_destroy(cigpu_crs *crs) {
    if (!crs) return CIGPU_OK;
    if (crs->stream) cudaStreamSynchronize(crs->stream);
    {
        StreamScope scope(crs->stream);  // blocks return to the cache ordered on this stream
        const bool own = crs->own_stream;
        cudaStream_t st = crs->stream;
        crs->own_stream = false;
        delete crs;
        if (own) cudaStreamDestroy(st);
    }
    return CIGPU_OK;
}

int cigpu_crs_dims(const cigpu_crs *crs, int64_t *dim, int64_t *nnz_upper, int64_t *nnz_full) {
    if (!crs) return CIGPU_EINVAL;
    if (nnz_upper || nnz_full) {  // the counts of a deferred build pass (the handle's lazily read state)
        CIGPU_TRY
        finish_deferred(*const_cast<cigpu_crs *>(crs));
        CIGPU_CATCH
    }
    if (dim) *dim = crs->dim;
    if (nnz_upper) *nnz_upper = crs->nnz_upper;
    if (nnz_full) *nnz_full = crs->nnz_full;
    return CIGPU_OK;
}

int cigpu_crs_layout(const cigpu_crs *crs, int *layout, int64_t *stored) {
    if (!crs) return CIGPU_EINVAL;
    if (layout)
        *layout = crs->onthefly ? CIGPU_LAYOUT_ONTHEFLY
                  : crs->pairs  ? CIGPU_LAYOUT_PAIRS
                  : crs->slots  ? CIGPU_LAYOUT_SLOTS
                                : CIGPU_LAYOUT_CRS;
    if (stored)
        *stored = crs->pairs                           ? 0
                  : crs->onthefly                      ? (crs->det_block > 0 ? crs->nnz_full : 0)
                  : crs->slots                         ? slots_stored(crs->fp)
                                                       : crs->nnz_full;
    return CIGPU_OK;
}

int cigpu_crs_fp32_product(const cigpu_crs *crs, int *kind, int *rank, int *padded) {
    if (!crs) return CIGPU_EINVAL;
    const bool sig = crs->sig != nullptr;
    if (kind) *kind = sig ? CIGPU_FP32_SIGMA : CIGPU_FP32_STORED;
    if (rank) *rank = sig ? crs->sig->rank : 0;
    if (padded) *padded = sig ? crs->sig->R : 0;
    return CIGPU_OK;
}

int cigpu_crs_export_upper(cigpu_crs *crs, uint32_t *row, uint32_t *col, double *val) {
    if (!crs || !row || !col || !val) return CIGPU_EINVAL;
    if (crs->onthefly) return CIGPU_ENOTSUP;
    CIGPU_TRY
    finish_deferred(*crs);
    if (crs->nnz_upper > (int64_t)UINT32_MAX) return CIGPU_ENOTSUP;
    cudaStream_t s = crs->stream;
    StreamScope scope(s);
    const int64_t dim = crs->dim;
    ExplicitCrs ex;
    const bool gen = crs->slots || crs->pairs;  // no stored explicit CRS: generate it
    if (gen) ex.make(*crs, s);
    DevBuf<uint32_t> ucnt(dim);
    DevBuf<int64_t> urow(dim + 1);
    upper_counts_launch(dim, crs->row_ptr.p, crs->upper_off.p, ucnt.p, s);
    exclusive_scan_u32(ucnt.p, urow.p, dim, s);
    DevBuf<uint32_t> ucol(crs->nnz_upper > 0 ? crs->nnz_upper : 1);
    DevBuf<double> uval(crs->nnz_upper > 0 ? crs->nnz_upper : 1);
    const bool f64 = crs->precision == CIGPU_FP64;
    extract_upper_launch(dim, crs->row_ptr.p, crs->upper_off.p, gen ? ex.col.p : crs->col.p,
                         f64 ? (gen ? ex.v64.p : crs->val64.p) : nullptr,
                         f64 ? nullptr : (gen ? ex.hi.p : crs->val32.p), urow.p, ucol.p, uval.p, s);
    std::vector<int64_t> hr(dim + 1);
    CIGPU_CUDA(cudaMemcpyAsync(hr.data(), urow.p, sizeof(int64_t) * (dim + 1), cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(col, ucol.p, sizeof(uint32_t) * crs->nnz_upper, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(val, uval.p, sizeof(double) * crs->nnz_upper, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
    for (int64_t i = 0; i <= dim; ++i) row[i] = (uint32_t)hr[i];
    return CIGPU_OK;
    CIGPU_CATCH
}

int cigpu_crs_export_full(cigpu_crs *crs, int64_t *row, uint32_t *col, double *val) {
    if (!crs || !row || !col || !val) return CIGPU_EINVAL;
    if (crs->onthefly) return CIGPU_ENOTSUP;
    CIGPU_TRY
    finish_deferred(*crs);
    cudaStream_t s = crs->stream;
    StreamScope scope(s);
    ExplicitCrs ex;
    const bool gen = crs->slots || crs->pairs;  // no stored explicit CRS: generate it
    if (gen) ex.make(*crs, s);
    CIGPU_CUDA(cudaMemcpyAsync(row, crs->row_ptr.p, sizeof(int64_t) * (crs->dim + 1), cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaMemcpyAsync(col, gen ? ex.col.p : crs->col.p, sizeof(uint32_t) * crs->nnz_full,
                               cudaMemcpyDeviceToHost, s));
    if (crs->precision == CIGPU_FP64) {
        CIGPU_CUDA(cudaMemcpyAsync(val, gen ? ex.v64.p : crs->val64.p, sizeof(double) * crs->nnz_full,
                                   cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaStreamSynchronize(s));
    } else {
        std::vector<float> tmp(crs->nnz_full);
        CIGPU_CUDA(cudaMemcpyAsync(tmp.data(), gen ? ex.hi.p : crs->val32.p, sizeof(float) * crs->nnz_full,
                                   cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaStreamSynchronize(s));
        for (int64_t i = 0; i < crs->nnz_full; ++i) val[i] = tmp[i];
    }
    return CIGPU_OK;
    CIGPU_CATCH
}

int cigpu_mvprod(cigpu_crs *crs, const double *x, double *y, cigpu_stream stream) {
    if (!crs || !x || !y) return CIGPU_EINVAL;
    CIGPU_TRY
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : crs->stream;
    StreamScope scope(s);
    DevBuf<double> dx(crs->dim), dy(crs->dim);
    CIGPU_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * crs->dim, cudaMemcpyHostToDevice, s));
    crs_mv64(*crs, dx.p, dy.p, s);
    CIGPU_CUDA(cudaMemcpyAsync(y, dy.p, sizeof(double) * crs->dim, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
    return CIGPU_OK;
    CIGPU_CATCH
}

int cigpu_mvprod_device(cigpu_crs *crs, const void *x, void *y, int dtype, cigpu_stream stream) {
    if (!crs || !x || !y || (dtype != 0 && dtype != 1)) return CIGPU_EINVAL;
    if (dtype == 1 && crs->precision != CIGPU_MIXED) return CIGPU_EINVAL;
    CIGPU_TRY
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : crs->stream;
    StreamScope scope(s);
    if (dtype == 0)
        crs_mv64(*crs, static_cast<const double *>(x), static_cast<double *>(y), s);
    else
        crs_mv32(*crs, static_cast<const float *>(x), static_cast<float *>(y), s);
    return CIGPU_OK;
    CIGPU_CATCH
}

int cigpu_solve(cigpu_crs *crs, double tol, int64_t max_matvec, const double *c0, double *c_out,
                cigpu_solve_info *info) {
    if (!crs || !(tol > 0) || max_matvec < 0) return CIGPU_EINVAL;
    CIGPU_TRY
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = crs->stream;
    StreamScope scope(s);
    DevBuf<double> c(crs->dim);
    if (c0) CIGPU_CUDA(cudaMemcpyAsync(c.p, c0, sizeof(double) * crs->dim, cudaMemcpyHostToDevice, s));
    cigpu_solve_info inf{};
    const int st = solve_crs(*crs, tol, max_matvec, c.p, c0 != nullptr, inf);
    if (c_out) CIGPU_CUDA(cudaMemcpyAsync(c_out, c.p, sizeof(double) * crs->dim, cudaMemcpyDeviceToHost, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
    inf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (info) *info = inf;
    return st;
    CIGPU_CATCH
}

int cigpu_rdm(cigpu_crs *crs, const double *c, double *rdm1, double *aa, double *ab, double *bb) {
    if (!crs || !c) return CIGPU_EINVAL;
    if (crs->method == CIGPU_DETS && crs->L > 64) return CIGPU_ENOTSUP;
    CIGPU_TRY
    cudaStream_t s = crs->stream;
    StreamScope scope(s);
    DevBuf<double> dc(crs->dim);
    CIGPU_CUDA(cudaMemcpyAsync(dc.p, c, sizeof(double) * crs->dim, cudaMemcpyHostToDevice, s));
    crs_rdm(*crs, dc.p, rdm1, aa, ab, bb, s);
    CIGPU_CUDA(cudaStreamSynchronize(s));
    return CIGPU_OK;
    CIGPU_CATCH
}

}  // extern "C"
