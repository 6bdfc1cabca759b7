// Continuous-batching solve server (cigpu_server_*).
//
// The served analogue of CIFlow's orbital-optimisation loop, where every rotated
// Hamiltonian goes through set_ham -> build -> solve (SimulatedAnnealing.cpp:
// 72-86, 130-134; CIMethod::set_ham, CIMethod.cpp:117-126). Requests of uneven
// size arrive at any time; each is admitted when a worker slot is free and its
// device-memory estimate fits the HBM budget, so requests that arrive while
// others run join as capacity frees up. Every worker owns a CUDA stream; the
// admitted requests' builds, matvecs and solves overlap on the device, and all
// state (integrals, CRS, Krylov vectors) stays on the device until the request
// completes. Device blocks come from the library's caching allocator, so no
// request's cleanup synchronises the whole device.
//
// Admission is FIFO with bounded backfilling: a request that does not fit may be
// passed by later, smaller ones at most kMaxBypass times; after that nothing
// behind it is admitted until it fits.
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "crs.cuh"

namespace {

constexpr int kMaxBypass = 16;

double now_s() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

struct Request {
    uint64_t id = 0;
    cigpu_request r{};
    std::vector<double> h, eri, c0, rot;
    size_t bytes = 0;
    int64_t dim = 0;
    int status = CIGPU_OK;
    bool done = false, running = false;
    int bypassed = 0;
    bool cancel = false;
    double t_submit = 0, t_admit = 0, t_done = 0;
    cigpu_solve_info info{};
    std::vector<double> c, rdm1;
};

int64_t dim_of(int L, int nup, int ndown, int method) {
    return cigpu::space_dim(method, L, nup, ndown);
}

// Host validation of a request at submit: sizes, and the same integral checks as
// cigpu_ham_create, so a bad request is refused before it is queued.
int validate(const cigpu_request &q) {
    if (q.L < 1 || q.L > cigpu::kMaxL || q.nup < 0 || q.ndown < 0 || q.nup > q.L || q.ndown > q.L) return CIGPU_EINVAL;
    if (q.method != CIGPU_FCI && q.method != CIGPU_DOCI) return CIGPU_EINVAL;
    if (q.precision != CIGPU_FP64 && q.precision != CIGPU_MIXED) return CIGPU_EINVAL;
    if (q.method == CIGPU_DOCI && q.nup != q.ndown) return CIGPU_EINVAL;
    if (!q.h || !q.eri || !(q.tol > 0) || !std::isfinite(q.econst)) return CIGPU_EINVAL;
    if (cigpu::validate_integrals(q.L, q.h, q.eri, nullptr) != CIGPU_OK) return CIGPU_EINVAL;
    if (q.rot && cigpu::validate_rotation(q.L, q.rot) != CIGPU_OK) return CIGPU_EINVAL;
    const int64_t d = dim_of(q.L, q.nup, q.ndown, q.method);
    if (d < 1 || d > (int64_t)UINT32_MAX) return CIGPU_ENOTSUP;
    return CIGPU_OK;
}

}  // namespace

struct cigpu_server {
    int device = 0;
    size_t budget = 0;
    int max_inflight = 1, max_queue = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;  // waiting for admission
    std::deque<std::shared_ptr<Request>> ready;  // admitted, waiting for a worker
    std::map<uint64_t, std::shared_ptr<Request>> all;
    size_t in_use = 0;
    int inflight = 0;
    int64_t admitted = 0, completed = 0;
    uint64_t next_id = 1;
    bool stop = false;
    std::vector<std::thread> workers;

    // Moves admissible requests from the queue to the ready list (mu held).
    // A request that does not fit counts one bypass each time a later request is
    // admitted ahead of it; once one has been passed kMaxBypass times, nothing
    // behind it is admitted until it fits.
    void admit_locked() {
        std::vector<Request *> waiting;  // earlier requests of this pass that did not fit
        for (auto it = queue.begin(); it != queue.end() && inflight < max_inflight;) {
            auto &q = *it;
            if (in_use + q->bytes <= budget) {
                bool held = false;
                for (Request *w : waiting) held = held || w->bypassed >= kMaxBypass;
                if (held) break;
                for (Request *w : waiting) ++w->bypassed;
                in_use += q->bytes;
                ++inflight;
                ++admitted;
                q->t_admit = now_s();
                ready.push_back(q);
                it = queue.erase(it);
                cv_work.notify_one();
            } else {
                waiting.push_back(q.get());
                ++it;
            }
        }
    }

    void run(Request &q, cudaStream_t s) {
        {
            std::lock_guard<std::mutex> lock(mu);
            if (q.cancel) {
                q.status = CIGPU_ECANCELED;
                return;
            }
        }
        cigpu::StreamScope scope(s);  // released blocks are ordered on this worker's stream
        cigpu_ham *ham = nullptr;
        cigpu_crs *crs = nullptr;
        int st = cigpu_ham_create(q.r.L, q.r.nup, q.r.ndown, q.r.econst, q.h.data(), q.eri.data(), &ham);
        if (st == CIGPU_OK && !q.rot.empty()) {  // orbital rotation on the device
            cigpu_ham *rotated = nullptr;
            st = cigpu_ham_rotate(ham, q.rot.data(), s, &rotated);
            cigpu_ham_destroy(ham);
            ham = rotated;
        }
        // several requests run at once: the sigma FP32 product on any grid (half the
        // GPU work of the stored values' product on L=10 5a5b, where one solve alone
        // is faster with the stored values)
        if (st == CIGPU_OK) st = cigpu::build_handle(ham, q.r.method, q.r.precision, s, true, &crs, true);
        bool cancelled;
        {
            std::lock_guard<std::mutex> lock(mu);
            cancelled = q.cancel;
        }
        if (st == CIGPU_OK && !cancelled) {
            q.c.resize(q.dim);
            st = cigpu_solve(crs, q.r.tol, 0, q.c0.empty() ? nullptr : q.c0.data(), q.c.data(), &q.info);
            if ((st == CIGPU_OK || st == CIGPU_ENOCONV) && q.r.want_rdm) {
                q.rdm1.resize((size_t)2 * q.r.L * q.r.L);
                const int st2 = cigpu_rdm(crs, q.c.data(), q.rdm1.data(), nullptr, nullptr, nullptr);
                if (st2 != CIGPU_OK) st = st2;
            }
        }
        if (cancelled) st = CIGPU_ECANCELED;
        if (crs) cigpu_crs_destroy(crs);
        if (ham) cigpu_ham_destroy(ham);
        q.status = st;
    }

    void worker() {
        cudaSetDevice(device);
        cudaStream_t s = nullptr;
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        for (;;) {
            std::shared_ptr<Request> q;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv_work.wait(lock, [&] { return stop || !ready.empty(); });
                if (ready.empty()) break;
                q = ready.front();
                ready.pop_front();
                q->running = true;
            }
            run(*q, s);
            {
                std::lock_guard<std::mutex> lock(mu);
                q->running = false;
                q->done = true;
                q->t_done = now_s();
                in_use -= q->bytes;
                --inflight;
                ++completed;
                admit_locked();
            }
            cv_done.notify_all();
        }
        if (s) cudaStreamDestroy(s);
    }
};

extern "C" {

int cigpu_server_create(int device, size_t hbm_budget_bytes, int max_inflight, int max_queue, cigpu_server **out) {
    if (!out || max_inflight < 1 || max_queue < 1) return CIGPU_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return CIGPU_ECUDA;
    }
    std::unique_ptr<cigpu_server> srv(new cigpu_server);
    srv->device = device;
    srv->max_inflight = max_inflight;
    srv->max_queue = max_queue;
    if (hbm_budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        cudaSetDevice(device);
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return CIGPU_ECUDA;
        hbm_budget_bytes = (size_t)(0.8 * (double)fr);
    }
    srv->budget = hbm_budget_bytes;
    for (int i = 0; i < max_inflight; ++i) srv->workers.emplace_back(&cigpu_server::worker, srv.get());
    *out = srv.release();
    return CIGPU_OK;
}

int cigpu_server_submit(cigpu_server *srv, const cigpu_request *req, uint64_t *id) {
    if (!srv || !req || !id) return CIGPU_EINVAL;
    const int v = validate(*req);
    if (v != CIGPU_OK) return v;
    auto q = std::make_shared<Request>();
    q->r = *req;
    const size_t L = req->L;
    q->dim = dim_of(req->L, req->nup, req->ndown, req->method);
    q->h.assign(req->h, req->h + L * L);
    q->eri.assign(req->eri, req->eri + L * L * L * L);
    if (req->c0) q->c0.assign(req->c0, req->c0 + q->dim);
    if (req->rot) q->rot.assign(req->rot, req->rot + L * L);
    q->r.h = q->r.eri = q->r.c0 = q->r.rot = nullptr;
    q->bytes = cigpu::estimate_bytes(req->L, req->nup, req->ndown, req->method, req->precision);
    std::lock_guard<std::mutex> lock(srv->mu);
    if (q->bytes > srv->budget) return CIGPU_ENOMEM;  // can never fit
    if ((int)srv->queue.size() >= srv->max_queue) return CIGPU_EAGAIN;
    q->id = srv->next_id++;
    q->t_submit = now_s();
    srv->all[q->id] = q;
    srv->queue.push_back(q);
    srv->admit_locked();
    *id = q->id;
    return CIGPU_OK;
}

int cigpu_server_poll(cigpu_server *srv, uint64_t id, int wait_ms, cigpu_result *out, double *c_out, double *rdm1) {
    if (!srv) return CIGPU_EINVAL;
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->all.find(id);
    if (it == srv->all.end()) return CIGPU_ENOTFOUND;
    std::shared_ptr<Request> q = it->second;
    if (!q->done && wait_ms != 0) {
        auto pred = [&] { return q->done; };
        if (wait_ms < 0)
            srv->cv_done.wait(lock, pred);
        else
            srv->cv_done.wait_for(lock, std::chrono::milliseconds(wait_ms), pred);
    }
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->done = q->done;
        out->dim = q->dim;
        out->status = q->done ? q->status : CIGPU_OK;
        if (q->done) {
            out->info = q->info;
            out->queued_s = (q->t_admit > 0 ? q->t_admit : q->t_done) - q->t_submit;
            out->latency_s = q->t_done - q->t_submit;
        }
    }
    if (!q->done) return wait_ms > 0 ? CIGPU_ETIMEDOUT : CIGPU_OK;
    if (c_out && q->c.size() == (size_t)q->dim) std::memcpy(c_out, q->c.data(), sizeof(double) * q->dim);
    if (rdm1 && !q->rdm1.empty()) std::memcpy(rdm1, q->rdm1.data(), sizeof(double) * q->rdm1.size());
    srv->all.erase(it);
    return CIGPU_OK;
}

int cigpu_server_cancel(cigpu_server *srv, uint64_t id) {
    if (!srv) return CIGPU_EINVAL;
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->all.find(id);
    if (it == srv->all.end()) return CIGPU_ENOTFOUND;
    auto q = it->second;
    if (q->done) return CIGPU_OK;
    for (auto qi = srv->queue.begin(); qi != srv->queue.end(); ++qi)
        if ((*qi)->id == id) {  // not admitted yet: finish it right away
            srv->queue.erase(qi);
            q->status = CIGPU_ECANCELED;
            q->done = true;
            q->t_done = now_s();
            srv->cv_done.notify_all();
            return CIGPU_OK;
        }
    q->cancel = true;  // admitted: the worker stops before the solve
    return CIGPU_OK;
}

int cigpu_server_stats(cigpu_server *srv, int64_t *admitted, int64_t *completed, int64_t *inflight,
                       size_t *hbm_in_use) {
    if (!srv) return CIGPU_EINVAL;
    std::lock_guard<std::mutex> lock(srv->mu);
    if (admitted) *admitted = srv->admitted;
    if (completed) *completed = srv->completed;
    if (inflight) *inflight = srv->inflight;
    if (hbm_in_use) *hbm_in_use = srv->in_use;
    return CIGPU_OK;
}

int cigpu_server_destroy(cigpu_server *srv) {
    if (!srv) return CIGPU_OK;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
        for (auto &q : srv->queue) {
            q->status = CIGPU_ECANCELED;
            q->done = true;
        }
        srv->queue.clear();
        for (auto &kv : srv->all) kv.second->cancel = true;
    }
    srv->cv_work.notify_all();
    srv->cv_done.notify_all();
    for (auto &t : srv->workers) t.join();
    delete srv;
    return CIGPU_OK;
}

}  // extern "C"
