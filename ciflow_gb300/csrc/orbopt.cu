// Orbital optimisation on the device: Jacobi rotations of a Hamiltonian
// (cigpu_ham_jacobi), the DOCI pair scan (cigpu_doci_pair_scan) and the optimiser
// loops (cigpu_orbopt_*).
//
// The reference optimisers (SimulatedAnnealing.cpp:42-391, LocalMinimizer.cpp:23-280)
// are a set_ham -> solve loop: every step rotates two orbitals of the current
// Hamiltonian (OrbitalTransform::do_jacobi_rotation, OrbitalTransform.cpp:278-414),
// rebuilds the CRS and solves it from scratch. Here each step stays on the device:
//   * the Jacobi rotation is one kernel over the L^4 tensor that recomputes every
//     element from its canonical representative (<= 16 products where an index is
//     k or l, a copy elsewhere), so the result is exactly 8-fold symmetric and
//     carries the FP32 split the mixed build reads;
//   * each solve starts from the current eigenvector (warm start): an orbital
//     rotation by a small angle moves the ground state by O(angle);
//   * the DOCI local minimiser's scan of all L(L-1)/2 pairs (DensDOCI::find_min_angle
//     and calc_rotate, CIDens.cpp:1279-1464) is one warp per pair on the DOCI pair
//     matrices the RDM kernel leaves on the device;
//   * simulated annealing evaluates up to `speculate` proposals of the chain at once,
//     each on its own stream: proposals are drawn in chain order from their own
//     random stream and all rotate the current orbitals; walking them in order, a
//     rejection leaves the current orbitals unchanged, so the next proposal's solve
//     is already the one the sequential chain would do; after an acceptance the
//     later proposals are solved again from the new orbitals. The chain (accepted
//     steps, energies, final orbitals) is the same for every value of `speculate`.
// Random numbers: splitmix64 (Steele, Lea and Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014), one stream for proposals and one for the
// acceptance draws; the reference seeds std::mt19937 from std::random_device, so
// its runs are not reproducible and no stream can match it draw for draw.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <vector>

#include "crs.cuh"
#include "small_eigh.h"

namespace cigpu {

namespace {

constexpr int kJacThreads = 256;
constexpr int kScanWarps = 4;  // pairs per block of the scan kernel

struct Givens {
    int k, l;
    double c, s;
};

// Row x of the Givens unitary: new k = c k - s l, new l = s k + c l, others unchanged.
__device__ __forceinline__ int givens_row(int x, const Givens &g, int *idx, double *w) {
    if (x == g.k) {
        idx[0] = g.k;
        w[0] = g.c;
        idx[1] = g.l;
        w[1] = -g.s;
        return 2;
    }
    if (x == g.l) {
        idx[0] = g.k;
        w[0] = g.s;
        idx[1] = g.l;
        w[1] = g.c;
        return 2;
    }
    idx[0] = x;
    w[0] = 1.0;
    return 1;
}

__global__ void __launch_bounds__(kJacThreads) k_jacobi_eri(int L, Givens g, const double *__restrict__ in,
                                                            double *__restrict__ eri, float *__restrict__ hi,
                                                            float *__restrict__ lo) {
    const int64_t L1 = L, L2 = L1 * L1, L3 = L2 * L1, total = L2 * L2;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(idx / L3), q = (int)((idx / L2) % L1), r = (int)((idx / L1) % L1), s = (int)(idx % L1);
        // canonical representative (a >= b, c >= d, ab >= cd): all 8 permutations
        // evaluate the same expression, so the result is exactly symmetric
        int a = max(p, q), b = min(p, q), c = max(r, s), d = min(r, s);
        if (a * L + b < c * L + d) {
            int t = a;
            a = c;
            c = t;
            t = b;
            b = d;
            d = t;
        }
        int ia[2], ib[2], ic[2], id[2];
        double wa[2], wb[2], wc[2], wd[2];
        const int na = givens_row(a, g, ia, wa), nb = givens_row(b, g, ib, wb);
        const int nc = givens_row(c, g, ic, wc), nd = givens_row(d, g, id, wd);
        double v = 0;
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j)
                for (int m = 0; m < nc; ++m)
                    for (int n = 0; n < nd; ++n)
                        v = fma(wa[i] * wb[j] * wc[m] * wd[n], in[ia[i] * L3 + ib[j] * L2 + ic[m] * L1 + id[n]], v);
        eri[idx] = v;
        split_fp32(v, hi[idx], lo[idx]);
    }
}

__global__ void k_jacobi_h(int L, Givens g, const double *__restrict__ h, double *__restrict__ out) {
    const int L2 = L * L;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < L2; idx += gridDim.x * blockDim.x) {
        const int p = idx / L, q = idx - p * L;
        const int a = max(p, q), b = min(p, q);
        int ia[2], ib[2];
        double wa[2], wb[2];
        const int na = givens_row(a, g, ia, wa), nb = givens_row(b, g, ib, wb);
        double v = 0;
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j) v = fma(wa[i] * wb[j], h[ia[i] * L + ib[j]], v);
        out[idx] = v;
    }
}

// ---------------------------------------------------------------------------
// DOCI pair scan. In the reference's element notation T(a,b) = h_ab,
// V(a,b,c,d) = <ab|cd> = (ac|bd), P(a,b) = Gamma_ab(aa,bb), D(a,b) = Gamma_aa(ab,ab)
// (zero for a = b), the energy after rotating k and l by t is
//   E(t) = E_rest + C4 cos^4 + S4 sin^4 + C2 cos^2 + S2 sin^2 + 2 SC sin cos
//          + 2 C2S2 cos^2 sin^2 + 4 S3C cos sin^3 + 4 C3S cos^3 sin
// with the coefficients of DensDOCI::calc_rotate (CIDens.cpp:1389-1464); its first
// and second derivatives drive the Newton search of find_min_angle (:1279-1387).
struct PairTerms {
    double rest, c4, s4, c2, s2, sc, c2s2, s3c, c3s;
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ double pt_energy(const PairTerms &t, double th) {
    const double c = cos(th), s = sin(th);
    return t.rest + c * c * c * c * t.c4 + s * s * s * s * t.s4 + c * c * t.c2 + s * s * t.s2 + 2 * s * c * t.sc +
           2 * c * c * s * s * t.c2s2 + 4 * c * s * s * s * t.s3c + 4 * c * c * c * s * t.c3s;
}

// dE/dt and d2E/dt2 of the expression above, differentiated term by term
// (d(c^2 s^2) = 2cs(c^2 - s^2), d(c s^3) = 3c^2 s^2 - s^4, d(c^3 s) = c^4 - 3c^2 s^2).
__device__ double pt_gradient(const PairTerms &t, double th) {
    const double c = cos(th), s = sin(th), cc = c * c, ss = s * s, cs = c * s;
    return -4 * t.c4 * cc * cs + 4 * t.s4 * ss * cs + 2 * (t.s2 - t.c2) * cs + 2 * t.sc * (cc - ss) +
           4 * t.c2s2 * cs * (cc - ss) + 4 * t.s3c * (3 * cc * ss - ss * ss) + 4 * t.c3s * (cc * cc - 3 * cc * ss);
}

__device__ double pt_hessian(const PairTerms &t, double th) {
    const double c = cos(th), s = sin(th), cc = c * c, ss = s * s, cs = c * s;
    return 4 * t.c4 * (3 * cc * ss - cc * cc) + 4 * t.s4 * (3 * cc * ss - ss * ss) + 2 * (t.s2 - t.c2) * (cc - ss) -
           8 * t.sc * cs + 4 * t.c2s2 * (cc * cc - 6 * cc * ss + ss * ss) + 4 * t.s3c * (6 * cs * (cc - ss) - 4 * ss * cs) -
           4 * t.c3s * (4 * cc * cs + 6 * cs * (cc - ss));
}

// Newton-Raphson from `start` (find_min_angle): flips the start when the quadratic
// model goes uphill, at most 20 steps, stops when |dx| < 1e-12. Returns the angle;
// *is_min = hessian > 0 there.
__device__ double newton_min(const PairTerms &t, double start, bool *is_min) {
    double th = start;
    const double change = pt_gradient(t, th) * th + pt_hessian(t, th) * th * th / 2.0;
    if (change > 0) th = -th;
    for (int it = 0; it < 20; ++it) {
        const double dx = pt_gradient(t, th) / pt_hessian(t, th);
        th -= dx;
        if (fabs(dx) < 1e-12) break;
    }
    *is_min = pt_hessian(t, th) > 0;
    return th;
}

__global__ void __launch_bounds__(32 * kScanWarps) k_doci_pair_scan(int L, int N, const double *__restrict__ h,
                                                                    const double *__restrict__ eri,
                                                                    const double *__restrict__ Pm,
                                                                    const double *__restrict__ Dm,
                                                                    double *__restrict__ theta,
                                                                    double *__restrict__ energy,
                                                                    int32_t *__restrict__ found) {
    const int np = L * (L - 1) / 2;
    const int pair = blockIdx.x * kScanWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (pair >= np) return;
    int k = 0, rem = pair;
    while (rem >= L - 1 - k) {
        rem -= L - 1 - k;
        ++k;
    }
    const int l = k + 1 + rem;
    const int64_t L1 = L, L2 = L1 * L1, L3 = L2 * L1;
    auto T = [&](int a, int b) { return h[a * L + b]; };
    auto V = [&](int a, int b, int c, int d) { return eri[a * L3 + c * L2 + b * L1 + d]; };  // <ab|cd> = (ac|bd)
    auto P = [&](int a, int b) { return Pm[a * L + b]; };
    auto D = [&](int a, int b) { return Dm[a * L + b]; };
    const double f = 2.0 / (N - 1.0);
    double c2 = 0, s2 = 0, sc = 0, rest = 0;
    for (int a = lane; a < L; a += 32) {
        if (a == k || a == l) continue;
        const double xk = 2 * V(k, a, k, a) - V(k, a, a, k) + f * T(k, k);
        const double xl = 2 * V(l, a, l, a) - V(l, a, a, l) + f * T(l, l);
        c2 += 2 * V(k, k, a, a) * P(k, a) + 2 * V(l, l, a, a) * P(l, a) + 2 * xk * D(k, a) + 2 * xl * D(l, a);
        s2 += 2 * V(l, l, a, a) * P(k, a) + 2 * V(k, k, a, a) * P(l, a) + 2 * xk * D(l, a) + 2 * xl * D(k, a);
        sc += 2 * V(k, l, a, a) * (P(l, a) - P(k, a)) +
              2 * (2 * V(k, a, l, a) - V(k, a, a, l) + f * T(k, l)) * (D(l, a) - D(k, a));
        rest += f * T(a, a) * (P(a, a) + 2 * D(a, k) + 2 * D(a, l));
    }
    for (int ab = lane; ab < L * L; ab += 32) {
        const int a = ab / L, b = ab - a * L;
        if (a == k || a == l || b == k || b == l) continue;
        rest += f * (T(a, a) + T(b, b)) * D(a, b) + V(a, a, b, b) * P(a, b) + (2 * V(a, b, a, b) - V(a, b, b, a)) * D(a, b);
    }
    c2 = warp_sum(c2);
    s2 = warp_sum(s2);
    sc = warp_sum(sc);
    rest = warp_sum(rest);
    if (lane != 0) return;
    PairTerms t;
    t.c2 = f * (T(k, k) * P(k, k) + T(l, l) * P(l, l)) + c2;
    t.s2 = f * (T(l, l) * P(k, k) + T(k, k) * P(l, l)) + s2;
    t.sc = f * T(k, l) * (P(l, l) - P(k, k)) + sc;
    t.rest = 2 * f * (T(k, k) + T(l, l)) * D(k, l) + rest;
    const double Vkkkk = V(k, k, k, k), Vllll = V(l, l, l, l), Vkkll = V(k, k, l, l), Vklkl = V(k, l, k, l);
    const double Vklkk = V(k, l, k, k), Vklll = V(k, l, l, l);
    const double Pkk = P(k, k), Pll = P(l, l), Pkl = P(k, l), Dkl = D(k, l);
    t.c4 = Vkkkk * Pkk + Vllll * Pll + 2 * Vkkll * Pkl + 2 * (2 * Vklkl - Vkkll) * Dkl;
    t.s4 = Vkkkk * Pll + Vllll * Pkk + 2 * Vkkll * Pkl + 2 * (2 * Vklkl - Vkkll) * Dkl;
    t.c2s2 = (2 * Vkkll + Vklkl) * (Pkk + Pll) + (Vkkkk + Vllll - 2 * (Vklkl + Vkkll)) * Pkl +
             (Vkkkk + Vllll - 6 * Vkkll + 2 * Vklkl) * Dkl;
    t.s3c = Vklkk * Pll - Vklll * Pkk - (Vklkk - Vklll) * (Pkl + Dkl);
    t.c3s = Vklll * Pll - Vklkk * Pkk + (Vklkk - Vklll) * (Pkl + Dkl);
    // scan_orbitals (LocalMinimizer.cpp:89-118): start at 0.3, then 0.01 if that
    // ended on a maximum; keep minima with |theta| <= pi/2
    bool is_min = false;
    double th = newton_min(t, 0.3, &is_min);
    if (!is_min) th = newton_min(t, 0.01, &is_min);
    theta[pair] = th;
    energy[pair] = pt_energy(t, th);
    found[pair] = (is_min && fabs(th) <= M_PI / 2.0) ? 1 : 0;
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(sm_count() * 8, (n + kJacThreads - 1) / kJacThreads)); }

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// New Hamiltonian with orbitals k, l of `base` rotated by theta. host_copy: also
// fill the host tables (the FCI build reads them); otherwise only the device ones.
void jacobi_ham(const cigpu_ham &base, int k, int l, double theta, cigpu_ham &H, cudaStream_t s, bool host_copy) {
    const int L = base.L;
    const size_t L2 = (size_t)L * L, L4 = L2 * L2;
    H.L = L;
    H.nup = base.nup;
    H.ndown = base.ndown;
    H.econst = base.econst;
    H.d_eri.alloc(L4);
    H.d_eri_hi.alloc(L4);
    H.d_eri_lo.alloc(L4);
    H.d_h.alloc(L2);
    const Givens g{k, l, std::cos(theta), std::sin(theta)};
    k_jacobi_eri<<<grid_for((int64_t)L4), kJacThreads, 0, s>>>(L, g, base.d_eri.p, H.d_eri.p, H.d_eri_hi.p, H.d_eri_lo.p);
    k_jacobi_h<<<grid_for((int64_t)L2), kJacThreads, 0, s>>>(L, g, base.d_h.p, H.d_h.p);
    CIGPU_CUDA(cudaGetLastError());
    count_launch(2);
    H.host_valid = host_copy;
    if (host_copy) {
        H.h.resize(L2);
        H.eri.resize(L4);
        CIGPU_CUDA(cudaMemcpyAsync(H.h.data(), H.d_h.p, L2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        CIGPU_CUDA(cudaMemcpyAsync(H.eri.data(), H.d_eri.p, L4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    } else {
        H.h.clear();
        H.eri.clear();
    }
    CIGPU_CUDA(cudaStreamSynchronize(s));
}

// Device copy of a Hamiltonian (host tables copied when valid).
void clone_ham(const cigpu_ham &src, cigpu_ham &H, cudaStream_t s) {
    const size_t L2 = (size_t)src.L * src.L, L4 = L2 * L2;
    H.L = src.L;
    H.nup = src.nup;
    H.ndown = src.ndown;
    H.econst = src.econst;
    H.host_valid = src.host_valid;
    H.h = src.h;
    H.eri = src.eri;
    H.d_h.alloc(L2);
    H.d_eri.alloc(L4);
    H.d_eri_hi.alloc(L4);
    H.d_eri_lo.alloc(L4);
    CIGPU_CUDA(cudaMemcpyAsync(H.d_h.p, src.d_h.p, L2 * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(H.d_eri.p, src.d_eri.p, L4 * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(H.d_eri_hi.p, src.d_eri_hi.p, L4 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    CIGPU_CUDA(cudaMemcpyAsync(H.d_eri_lo.p, src.d_eri_lo.p, L4 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    CIGPU_CUDA(cudaStreamSynchronize(s));
}

// The scan of every pair of a DOCI state (device vector c) into device outputs.
void doci_pair_scan(cigpu_crs &crs, const double *c_dev, double *partial, double *Pm, double *Dm, double *theta,
                    double *energy, int32_t *found, cudaStream_t s) {
    doci_pair_matrices(crs, c_dev, partial, Pm, Dm, s);
    const int L = crs.L, np = L * (L - 1) / 2;
    if (np == 0) return;
    k_doci_pair_scan<<<(np + kScanWarps - 1) / kScanWarps, 32 * kScanWarps, 0, s>>>(
        L, crs.nup + crs.ndown, crs.ham->d_h.p, crs.ham->d_eri.p, Pm, Dm, theta, energy, found);
    CIGPU_CUDA(cudaGetLastError());
    count_launch();
}

namespace {

// splitmix64; uniform() in [0, 1) with 53 random bits, below(n) = floor(uniform() * n).
struct Rng {
    uint64_t s = 0;
    explicit Rng(uint64_t seed = 0) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    int below(int n) { return (int)(uniform() * n); }
};

// Seeds of the per-call proposal streams and of the acceptance stream.
uint64_t stream_seed(uint64_t seed, uint64_t tag) {
    Rng r(seed ^ (0xD1B54A32D192ED03ull * (tag + 1)));
    return r.next();
}

// A solved Hamiltonian: the integrals, their CRS and ground state.
struct State {
    std::unique_ptr<cigpu_ham> ham;
    std::unique_ptr<cigpu_crs> crs;
    DevBuf<double> c;
    cigpu_solve_info info{};
    int status = CIGPU_OK;
    double t_rotate = 0, t_build = 0, t_solve = 0;
};

// Persistent worker threads, one stream each, for the speculative solves.
class Pool {
   public:
    explicit Pool(int n) {
        for (int w = 0; w < n; ++w) {
            cudaStream_t s = nullptr;
            CIGPU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            streams_.push_back(s);
        }
        for (int w = 0; w < n; ++w) threads_.emplace_back([this, w] { loop(w); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : threads_) t.join();
        for (auto s : streams_) cudaStreamDestroy(s);
    }
    int size() const { return (int)streams_.size(); }
    // Runs job(stream, j) for j in [0, n) on the workers; returns when all are done.
    void run(int n, const std::function<void(cudaStream_t, int)> &job) {
        std::unique_lock<std::mutex> lk(m_);
        job_ = &job;
        njobs_ = n;
        next_ = 0;
        done_ = 0;
        ++gen_;
        cv_.notify_all();
        done_cv_.wait(lk, [&] { return done_ == njobs_; });
        job_ = nullptr;
    }

   private:
    void loop(int w) {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(m_);
        for (;;) {
            cv_.wait(lk, [&] { return stop_ || (gen_ != seen && next_ < njobs_); });
            if (stop_) return;
            while (next_ < njobs_) {
                const int j = next_++;
                const auto *job = job_;
                lk.unlock();
                (*job)(streams_[w], j);
                lk.lock();
                if (++done_ == njobs_) done_cv_.notify_all();
            }
            seen = gen_;
        }
    }
    std::vector<cudaStream_t> streams_;
    std::vector<std::thread> threads_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(cudaStream_t, int)> *job_ = nullptr;
    int njobs_ = 0, next_ = 0, done_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

}  // namespace

}  // namespace cigpu

using namespace cigpu;

struct cigpu_orbopt {
    cigpu_orbopt_config cfg{};
    int L = 0;
    int64_t dim = 0;
    cudaStream_t s = nullptr;
    std::unique_ptr<cigpu_ham> base;
    State cur;
    std::vector<double> U, Uopt;
    double e_opt = 0;
    cigpu_orbopt_stats st{};
    uint64_t anneal_calls = 0;
    Rng acc;
    std::unique_ptr<Pool> pool;
    // DOCI scan scratch
    DevBuf<double> partial, Pm, Dm, theta, energy;
    DevBuf<int32_t> found;

    ~cigpu_orbopt() {
        {
            StreamScope scope(s);
            cur = State{};
            base.reset();
            partial.release();
            Pm.release();
            Dm.release();
            theta.release();
            energy.release();
            found.release();
            if (s) cudaStreamSynchronize(s);
        }
        pool.reset();
        if (s) cudaStreamDestroy(s);
    }

    bool host_tables() const { return cfg.method == CIGPU_FCI; }

    // Builds and solves `ham` (owned by out) on stream s; c0: optional device start.
    void solve_into(State &out, std::unique_ptr<cigpu_ham> ham, const double *c0, cudaStream_t ss) {
        const auto t0 = std::chrono::steady_clock::now();
        out.ham = std::move(ham);
        out.crs.reset(new cigpu_crs);
        cigpu_crs &c = *out.crs;
        c.ham = out.ham.get();
        c.method = cfg.method;
        c.precision = cfg.precision;
        c.L = L;
        c.nup = out.ham->nup;
        c.ndown = out.ham->ndown;
        c.dim = dim;
        c.stream = ss;
        c.own_stream = false;
        build_crs(c, ss);
        CIGPU_CUDA(cudaStreamSynchronize(ss));
        const auto t1 = std::chrono::steady_clock::now();
        out.t_build = std::chrono::duration<double>(t1 - t0).count();
        out.c.alloc(dim);
        if (c0) CIGPU_CUDA(cudaMemcpyAsync(out.c.p, c0, sizeof(double) * dim, cudaMemcpyDeviceToDevice, ss));
        out.status = solve_crs(c, cfg.tol, 0, out.c.p, c0 != nullptr, out.info, ss);
        CIGPU_CUDA(cudaStreamSynchronize(ss));
        out.t_solve = seconds_since(t1);
    }

    // Jacobi-rotated current Hamiltonian, solved (warm start from the current vector).
    void evaluate(State &out, int k, int l, double angle, cudaStream_t ss) {
        const auto t0 = std::chrono::steady_clock::now();
        std::unique_ptr<cigpu_ham> H(new cigpu_ham);
        jacobi_ham(*cur.ham, k, l, angle, *H, ss, host_tables());
        const double tr = seconds_since(t0);
        solve_into(out, std::move(H), cfg.warm_start ? cur.c.p : nullptr, ss);
        out.t_rotate = tr;
    }

    // Fully rotated Hamiltonian from the start orbitals, solved from scratch.
    void rotate_and_solve(State &out, const std::vector<double> &u) {
        const auto t0 = std::chrono::steady_clock::now();
        std::unique_ptr<cigpu_ham> H(new cigpu_ham);
        rotate_ham(*base, u.data(), *H, s);
        const double tr = seconds_since(t0);
        solve_into(out, std::move(H), nullptr, s);
        out.t_rotate = tr;
    }

    void account(const State &x) {
        ++st.solves;
        st.matvecs_fp64 += x.info.matvecs_fp64;
        st.matvecs_fp32 += x.info.matvecs_fp32;
        st.seconds_rotate += x.t_rotate;
        st.seconds_build += x.t_build;
        st.seconds_solve += x.t_solve;
    }

    static int ok(int status) { return status == CIGPU_OK || status == CIGPU_ENOCONV; }

    // UnitaryMatrix::jacobi_rotation: rows k and l of U.
    void jacobi_unitary(int k, int l, double angle) {
        const double c = std::cos(angle), s_ = std::sin(angle);
        for (int p = 0; p < L; ++p) {
            const double uk = U[(size_t)k * L + p], ul = U[(size_t)l * L + p];
            U[(size_t)k * L + p] = c * uk - s_ * ul;
            U[(size_t)l * L + p] = c * ul + s_ * uk;
        }
    }

    void scan_scratch() {
        if (partial.p) return;
        const size_t L2 = (size_t)L * L, np = std::max<size_t>(1, L2 / 2);
        partial.alloc((size_t)doci_pair_partials() * 2 * L2);
        Pm.alloc(L2);
        Dm.alloc(L2);
        theta.alloc(np);
        energy.alloc(np);
        found.alloc(np);
    }
};

namespace {

struct Proposal {
    int k, l;
    double angle, temp, max_angle_after;
};

int anneal(cigpu_orbopt &o, const cigpu_anneal_params &p, double *e_last) {
    const int K = std::max(1, std::min(p.speculate, 64));
    if (K > 1 && (!o.pool || o.pool->size() < K)) o.pool.reset(new Pool(K));
    Rng prop(stream_seed(o.cfg.seed, 2 * o.anneal_calls + 1));
    ++o.anneal_calls;
    const int L = o.L;
    double temp = p.temp, max_angle = p.max_angle;
    double e_old = o.cur.info.e0;  // cost_function(): the current energy
    int64_t ll = 0, unaccept = 0;
    std::deque<Proposal> pending;
    // draws the next proposals of the chain: rani, ranj uniform over the orbitals
    // (one irrep in C1); rani == ranj uses a loop iteration and no decay
    auto draw = [&](size_t want) {
        while (pending.size() < want && ll < p.steps) {
            const int i = prop.below(L), j = prop.below(L);
            ++ll;
            if (i == j) continue;
            Proposal q;
            q.k = i;
            q.l = j;
            const double u1 = prop.uniform(), u2 = prop.uniform();
            q.angle = max_angle * (u1 - u2);
            q.temp = temp;
            temp *= p.change_temp;
            max_angle *= p.change_angle;
            q.max_angle_after = max_angle;
            pending.push_back(q);
        }
    };
    std::vector<State> cand(K);
    bool stop = false;
    // Proposals per round: about 1 / (recent acceptance rate), at most K. A round
    // ends at its first acceptance, so at rate p it uses ~1/p of its proposals.
    double rate = 0.5;
    while (!stop) {
        const int want = std::max(1, std::min(K, (int)std::floor(1.0 / std::max(rate, 1e-3))));
        draw((size_t)want);
        if (pending.empty()) break;
        const int m = (int)std::min<size_t>(want, pending.size());
        std::vector<const Proposal *> batch;
        for (int j = 0; j < m; ++j) batch.push_back(&pending[j]);
        if (m == 1) {
            o.evaluate(cand[0], batch[0]->k, batch[0]->l, batch[0]->angle, o.s);
        } else {
            o.pool->run(m, [&](cudaStream_t ws, int j) {
                StreamScope scope(ws);
                try {
                    o.evaluate(cand[j], batch[j]->k, batch[j]->l, batch[j]->angle, ws);
                } catch (...) {
                    cand[j].status = status_from_exception();
                }
            });
        }
        for (int j = 0; j < m; ++j) o.account(cand[j]);
        for (int j = 0; j < m; ++j) {
            const Proposal q = pending.front();
            pending.pop_front();
            State &c = cand[j];
            if (!cigpu_orbopt::ok(c.status)) return c.status;
            const double e_new = c.info.e0;
            bool accept = true;
            if (!(e_new < e_old)) {
                // accept_function (SimulatedAnnealing.cpp:274-296)
                const double cost = std::exp((e_old - e_new) / q.temp);
                accept = !(o.acc.uniform() * (1 + cost) > cost);
            }
            ++o.st.steps;
            rate = 0.9 * rate + (accept ? 0.1 : 0.0);
            if (accept) {
                ++o.st.accepted;
                e_old = e_new;
                o.jacobi_unitary(q.k, q.l, q.angle);
                o.cur = std::move(c);
                o.cur.crs->stream = o.s;  // the worker stream stays with the pool
                if (e_new < o.e_opt) {
                    o.e_opt = e_new;
                    o.Uopt = o.U;
                }
                unaccept = 0;
            } else {
                ++o.st.rejected;
                ++unaccept;
            }
            if (unaccept > p.max_unaccept || q.max_angle_after < p.min_angle) {
                o.st.speculative_waste += m - 1 - j;
                stop = true;
                break;
            }
            if (accept) {
                o.st.speculative_waste += m - 1 - j;
                break;
            }
        }
        for (auto &c : cand) c = State{};
    }
    if (e_last) *e_last = e_old;
    return CIGPU_OK;
}

int local_min(cigpu_orbopt &o, const cigpu_local_params &p, double *e_final) {
    if (o.cfg.method != CIGPU_DOCI) return CIGPU_ENOTSUP;
    const int L = o.L, np = L * (L - 1) / 2;
    o.scan_scratch();
    std::vector<double> th(np), en(np);
    std::vector<int32_t> fd(np);
    struct Rot {
        int k, l;
        double angle, e;
    };
    int converged = 0, iters = 1;
    double opt_energy = 0;  // LocalMinimizer::optimize starts _opt_energy at 0
    std::pair<int, int> prev(0, 0);
    auto choose = [&](const std::vector<Rot> &rots) {
        // choose_orbitalpair (LocalMinimizer.cpp:258-280): weights opt_energy - e
        const double u = o.acc.uniform();
        double norm = 0, cum = 0;
        for (const auto &r : rots) norm += opt_energy - r.e;
        for (size_t i = 0; i < rots.size(); ++i) {
            cum += (opt_energy - rots[i].e) / norm;
            if (u < cum) return (int)i;
        }
        return (int)rots.size() - 1;
    };
    while (converged < p.conv_steps) {
        const auto t0 = std::chrono::steady_clock::now();
        doci_pair_scan(*o.cur.crs, o.cur.c.p, o.partial.p, o.Pm.p, o.Dm.p, o.theta.p, o.energy.p, o.found.p, o.s);
        CIGPU_CUDA(cudaMemcpyAsync(th.data(), o.theta.p, sizeof(double) * np, cudaMemcpyDeviceToHost, o.s));
        CIGPU_CUDA(cudaMemcpyAsync(en.data(), o.energy.p, sizeof(double) * np, cudaMemcpyDeviceToHost, o.s));
        CIGPU_CUDA(cudaMemcpyAsync(fd.data(), o.found.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, o.s));
        CIGPU_CUDA(cudaStreamSynchronize(o.s));
        o.st.seconds_scan += seconds_since(t0);
        std::vector<Rot> rots;
        int pi = 0;
        for (int k = 0; k < L; ++k)
            for (int l = k + 1; l < L; ++l, ++pi)
                if (fd[pi]) rots.push_back(Rot{k, l, th[pi], en[pi]});
        if (rots.empty()) return CIGPU_ENOCONV;
        std::stable_sort(rots.begin(), rots.end(), [](const Rot &a, const Rot &b) { return a.e < b.e; });
        int idx = 0;
        auto pair_of = [&](int i) { return std::make_pair(rots[i].k, rots[i].l); };
        if (p.dist_choice) {
            idx = choose(rots);
            if (pair_of(idx) == prev) idx = choose(rots);
            if (pair_of(idx) == prev) idx = 0;
        }
        // never the same pair twice in a row (a one-pair list has no alternative)
        if (pair_of(idx) == prev && (size_t)idx + 1 < rots.size()) ++idx;
        const Rot r = rots[idx];
        prev = pair_of(idx);
        State next;
        o.evaluate(next, r.k, r.l, r.angle, o.s);
        o.account(next);
        if (!cigpu_orbopt::ok(next.status)) return next.status;
        o.jacobi_unitary(r.k, r.l, r.angle);
        o.cur = std::move(next);
        ++o.st.steps;
        const double E = o.cur.info.e0;
        if (std::fabs(opt_energy - E) < p.conv_crit) ++converged;
        opt_energy = E;
        ++iters;
        if (iters > p.max_iters) break;
    }
    o.e_opt = opt_energy;
    o.Uopt = o.U;
    if (e_final) *e_final = o.cur.info.e0;
    return CIGPU_OK;
}

}  // namespace

extern "C" {

int cigpu_ham_jacobi(const cigpu_ham *base, int k, int l, double theta, cigpu_stream stream, cigpu_ham **out) {
    if (!base || !out) return CIGPU_EINVAL;
    *out = nullptr;
    if (k < 0 || l < 0 || k >= base->L || l >= base->L || k == l || !std::isfinite(theta)) return CIGPU_EINVAL;
    try {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        bool own = false;
        if (!s) {
            CIGPU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            own = true;
        }
        std::unique_ptr<std::remove_pointer_t<cudaStream_t>, decltype(&cudaStreamDestroy)> sg(own ? s : nullptr,
                                                                                             cudaStreamDestroy);
        std::unique_ptr<cigpu_ham> H(new cigpu_ham);
        {
            StreamScope scope(s);
            jacobi_ham(*base, k, l, theta, *H, s, true);
        }
        *out = H.release();
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_doci_pair_scan(cigpu_crs *crs, const double *c, double *theta, double *energy, int32_t *found) {
    if (!crs || !c || !theta || !energy || !found) return CIGPU_EINVAL;
    if (crs->method != CIGPU_DOCI) return CIGPU_EINVAL;
    if (crs->L > 32) return CIGPU_ENOTSUP;
    try {
        cudaStream_t s = crs->stream;
        StreamScope scope(s);
        const int L = crs->L, np = L * (L - 1) / 2;
        const size_t L2 = (size_t)L * L;
        DevBuf<double> dc(crs->dim), partial((size_t)doci_pair_partials() * 2 * L2), Pm(L2), Dm(L2);
        DevBuf<double> dth(std::max(np, 1)), den(std::max(np, 1));
        DevBuf<int32_t> dfd(std::max(np, 1));
        CIGPU_CUDA(cudaMemcpyAsync(dc.p, c, sizeof(double) * crs->dim, cudaMemcpyHostToDevice, s));
        doci_pair_scan(*crs, dc.p, partial.p, Pm.p, Dm.p, dth.p, den.p, dfd.p, s);
        if (np > 0) {
            CIGPU_CUDA(cudaMemcpyAsync(theta, dth.p, sizeof(double) * np, cudaMemcpyDeviceToHost, s));
            CIGPU_CUDA(cudaMemcpyAsync(energy, den.p, sizeof(double) * np, cudaMemcpyDeviceToHost, s));
            CIGPU_CUDA(cudaMemcpyAsync(found, dfd.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, s));
        }
        CIGPU_CUDA(cudaStreamSynchronize(s));
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_create(const cigpu_ham *ham, const cigpu_orbopt_config *cfg, cigpu_orbopt **out) {
    if (!ham || !cfg || !out) return CIGPU_EINVAL;
    *out = nullptr;
    if (cfg->method != CIGPU_FCI && cfg->method != CIGPU_DOCI) return CIGPU_EINVAL;
    if (cfg->precision != CIGPU_FP64 && cfg->precision != CIGPU_MIXED) return CIGPU_EINVAL;
    if (!(cfg->tol > 0)) return CIGPU_EINVAL;
    if (cfg->method == CIGPU_DOCI && (ham->nup != ham->ndown || ham->L > 32)) return CIGPU_ENOTSUP;
    if (cfg->method == CIGPU_FCI && !ham->host_valid) return CIGPU_EINVAL;
    if (ham->L > kMaxL) return CIGPU_ENOTSUP;
    const int64_t dim = space_dim(cfg->method, ham->L, ham->nup, ham->ndown);
    if (dim < 1 || dim > (int64_t)UINT32_MAX) return CIGPU_ENOTSUP;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        std::unique_ptr<cigpu_orbopt> o(new cigpu_orbopt);
        o->cfg = *cfg;
        o->L = ham->L;
        o->dim = dim;
        CIGPU_CUDA(cudaStreamCreateWithFlags(&o->s, cudaStreamNonBlocking));
        StreamScope scope(o->s);
        o->base.reset(new cigpu_ham);
        clone_ham(*ham, *o->base, o->s);
        o->U.assign((size_t)o->L * o->L, 0.0);
        for (int i = 0; i < o->L; ++i) o->U[(size_t)i * o->L + i] = 1.0;
        o->Uopt = o->U;
        std::unique_ptr<cigpu_ham> H(new cigpu_ham);
        clone_ham(*o->base, *H, o->s);
        o->solve_into(o->cur, std::move(H), nullptr, o->s);
        o->account(o->cur);
        if (!cigpu_orbopt::ok(o->cur.status)) return o->cur.status;
        o->e_opt = o->cur.info.e0;
        o->acc = Rng(stream_seed(cfg->seed, 0));
        o->st.seconds += seconds_since(t0);
        *out = o.release();
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_destroy(cigpu_orbopt *opt) {
    delete opt;
    return CIGPU_OK;
}

int cigpu_orbopt_anneal(cigpu_orbopt *opt, const cigpu_anneal_params *p, double *e_last) {
    if (!opt || !p) return CIGPU_EINVAL;
    if (!(p->temp > 0) || !(p->change_temp > 0) || !std::isfinite(p->max_angle) || !(p->change_angle > 0) ||
        p->steps < 0 || p->max_unaccept < 0 || p->speculate < 1)
        return CIGPU_EINVAL;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        StreamScope scope(opt->s);
        const int st = anneal(*opt, *p, e_last);
        opt->st.seconds += seconds_since(t0);
        return st;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_local(cigpu_orbopt *opt, const cigpu_local_params *p, double *e_final) {
    if (!opt || !p) return CIGPU_EINVAL;
    if (!(p->conv_crit >= 0) || p->conv_steps < 0 || p->max_iters < 1) return CIGPU_EINVAL;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        StreamScope scope(opt->s);
        const int st = local_min(*opt, *p, e_final);
        opt->st.seconds += seconds_since(t0);
        return st;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_jacobi(cigpu_orbopt *opt, int k, int l, double theta, double *e) {
    if (!opt) return CIGPU_EINVAL;
    if (k < 0 || l < 0 || k >= opt->L || l >= opt->L || k == l || !std::isfinite(theta)) return CIGPU_EINVAL;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        StreamScope scope(opt->s);
        State next;
        opt->evaluate(next, k, l, theta, opt->s);
        opt->account(next);
        if (!cigpu_orbopt::ok(next.status)) return next.status;
        opt->jacobi_unitary(k, l, theta);
        opt->cur = std::move(next);
        if (e) *e = opt->cur.info.e0;
        opt->st.seconds += seconds_since(t0);
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_natural(cigpu_orbopt *opt, int density_method, double *e) {
    if (!opt) return CIGPU_EINVAL;
    if (density_method != CIGPU_FCI && density_method != CIGPU_DOCI) return CIGPU_EINVAL;
    if (density_method == CIGPU_DOCI && opt->cur.ham->nup != opt->cur.ham->ndown) return CIGPU_EINVAL;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        StreamScope scope(opt->s);
        const int L = opt->L;
        const size_t L2 = (size_t)L * L;
        std::vector<double> rdm1(2 * L2);
        if (density_method == opt->cfg.method) {
            crs_rdm(*opt->cur.crs, opt->cur.c.p, rdm1.data(), nullptr, nullptr, nullptr, opt->s);
        } else {
            // get_fci_no: the FCI ground state of the current orbitals (FP64)
            if (density_method == CIGPU_FCI && !opt->cur.ham->host_valid) {
                opt->cur.ham->h.resize(L2);
                opt->cur.ham->eri.resize(L2 * L2);
                CIGPU_CUDA(cudaMemcpyAsync(opt->cur.ham->h.data(), opt->cur.ham->d_h.p, L2 * sizeof(double),
                                           cudaMemcpyDeviceToHost, opt->s));
                CIGPU_CUDA(cudaMemcpyAsync(opt->cur.ham->eri.data(), opt->cur.ham->d_eri.p, L2 * L2 * sizeof(double),
                                           cudaMemcpyDeviceToHost, opt->s));
                CIGPU_CUDA(cudaStreamSynchronize(opt->s));
                opt->cur.ham->host_valid = true;
            }
            cigpu_crs c;
            c.ham = opt->cur.ham.get();
            c.method = density_method;
            c.precision = CIGPU_FP64;
            c.L = L;
            c.nup = c.ham->nup;
            c.ndown = c.ham->ndown;
            c.dim = space_dim(density_method, L, c.nup, c.ndown);
            c.stream = opt->s;
            build_crs(c, opt->s);
            DevBuf<double> v(c.dim);
            cigpu_solve_info info{};
            const int st = solve_crs(c, opt->cfg.tol, 0, v.p, false, info, opt->s);
            if (!cigpu_orbopt::ok(st)) return st;
            crs_rdm(c, v.p, rdm1.data(), nullptr, nullptr, nullptr, opt->s);
        }
        // CIDens::get_no (CIDens.cpp:488-530): eigenvectors of the spin-summed 1-RDM,
        // natural orbital i = eigenvector of the i-th largest occupation
        std::vector<double> a(L2), w, z;
        for (size_t i = 0; i < L2; ++i) a[i] = rdm1[i] + rdm1[L2 + i];
        symmetric_eigh(L, a, w, z);
        // rotate_active_space_vectors (UnitaryMatrix.cpp:367-407): U <- NO^T U
        std::vector<double> Un(L2, 0.0);
        for (int i = 0; i < L; ++i) {
            const int col = L - 1 - i;
            for (int j = 0; j < L; ++j) {
                const double nij = z[(size_t)j * L + col];
                for (int p = 0; p < L; ++p) Un[(size_t)i * L + p] += nij * opt->U[(size_t)j * L + p];
            }
        }
        opt->U = Un;
        State next;
        opt->rotate_and_solve(next, opt->U);
        opt->account(next);
        if (!cigpu_orbopt::ok(next.status)) return next.status;
        opt->cur = std::move(next);
        if (e) *e = opt->cur.info.e0;
        opt->st.seconds += seconds_since(t0);
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_set_optimal(cigpu_orbopt *opt) {
    if (!opt) return CIGPU_EINVAL;
    try {
        const auto t0 = std::chrono::steady_clock::now();
        StreamScope scope(opt->s);
        opt->U = opt->Uopt;
        State next;
        opt->rotate_and_solve(next, opt->U);
        opt->account(next);
        if (!cigpu_orbopt::ok(next.status)) return next.status;
        opt->cur = std::move(next);
        opt->st.seconds += seconds_since(t0);
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_get(const cigpu_orbopt *opt, double *U, double *U_opt, double *c, cigpu_orbopt_stats *stats) {
    if (!opt) return CIGPU_EINVAL;
    try {
        if (U) std::memcpy(U, opt->U.data(), sizeof(double) * opt->U.size());
        if (U_opt) std::memcpy(U_opt, opt->Uopt.data(), sizeof(double) * opt->Uopt.size());
        if (c) {
            CIGPU_CUDA(cudaMemcpyAsync(c, opt->cur.c.p, sizeof(double) * opt->dim, cudaMemcpyDeviceToHost, opt->s));
            CIGPU_CUDA(cudaStreamSynchronize(opt->s));
        }
        if (stats) {
            *stats = opt->st;
            stats->e_current = opt->cur.info.e0;
            stats->e_opt = opt->e_opt;
        }
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

int cigpu_orbopt_ham(const cigpu_orbopt *opt, cigpu_ham **out) {
    if (!opt || !out) return CIGPU_EINVAL;
    *out = nullptr;
    try {
        StreamScope scope(opt->s);
        std::unique_ptr<cigpu_ham> H(new cigpu_ham);
        clone_ham(*opt->cur.ham, *H, opt->s);
        if (!H->host_valid) {
            const size_t L2 = (size_t)H->L * H->L;
            H->h.resize(L2);
            H->eri.resize(L2 * L2);
            CIGPU_CUDA(cudaMemcpyAsync(H->h.data(), H->d_h.p, L2 * sizeof(double), cudaMemcpyDeviceToHost, opt->s));
            CIGPU_CUDA(
                cudaMemcpyAsync(H->eri.data(), H->d_eri.p, L2 * L2 * sizeof(double), cudaMemcpyDeviceToHost, opt->s));
            CIGPU_CUDA(cudaStreamSynchronize(opt->s));
            H->host_valid = true;
        }
        *out = H.release();
        return CIGPU_OK;
    } catch (...) {
        return status_from_exception();
    }
}

}  // extern "C"
