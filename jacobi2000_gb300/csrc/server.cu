// Serving loop: continuous batching of forward, rewind and reconstruct
// requests of different grid sizes on one GPU.
//
// A server thread runs iterations. An iteration admits waiting requests, then
// runs a chunk of K ticks for every active request without returning to the
// host in between, then collects the requests that finished. Per tick, all
// instances that use the forward weights go into one packed launch sequence
// and all that use the reverse weights into another:
//   forward     request: its state (one instance, forward model), projected;
//   rewind      request: its state (one instance, reverse model), projected
//               (the web demo's rewind, crates/web/src/lib.rs:383-409);
//   reconstruct request: one Jacobi sweep of its space-time volume X[0..H]:
//               F_t = step_F(X_{t-1}) for t = 1..H (forward model) and
//               R_t = step_R(X_{t+1}) for t = 0..H-1 (reverse model), then
//               X_t <- known_t ? value : average of the available F_t, R_t,
//               until the largest change of an unknown value is below `tol`
//               or `max_sweeps` sweeps ran, without projection. This task has no
//               counterpart in the reference (its tests pin it against the
//               oracle restated with the same rule).
// Within a chunk each group's instances are ordered by the ticks (sweeps) they
// have left, longest first, so the instances still running at chunk tick t
// are a prefix: a request that finishes inside the chunk simply drops out of
// the later ticks' launches. A reconstruct request that converges inside the
// chunk is frozen on the device (its volume no longer changes). The chunk
// ends early when a waiting request could be admitted, or after about
// kChunkTargetS of device time when nothing waits.
// Requests that arrive while a chunk runs are admitted at the next iteration,
// while their instances fit the workspace and their buffers fit the device
// memory budget; each request's state stays on the device until jc_server_wait
// has copied its result out.
// A request is staged at submit when the budget has room (its buffers
// reserved and its inputs copied on a separate copy stream while chunks
// run), so that admitting it costs the next chunk an event wait, not the
// copies.
// A request's result does not depend on which other requests share its
// launches (no kernel's arithmetic for one instance reads another's data),
// nor on how its ticks are cut into chunks.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include "bf16_path.hpp"
#include "runtime.hpp"

namespace jc {

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Longest chunk when nothing waits: about this much device time.
constexpr double kChunkTargetS = 4e-3;
constexpr int kMaxChunk = 64;

// X_t <- known_t ? value : 0 (the normalized mean state) for every t. Work
// unit = (time slice, block of blockDim.x cells): a CTA takes units with
// stride gridDim.x, a thread one cell of the unit and its three channels.
__global__ void recon_fill_kernel(float* __restrict__ vol, const float* __restrict__ vals,
                                  const uint8_t* __restrict__ known, int H, long long cells) {
    const long long per = 3 * cells, ncb = (cells + blockDim.x - 1) / blockDim.x;
    const long long units = (long long)(H + 1) * ncb;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const long long t = u / ncb, cell = (u - t * ncb) * blockDim.x + threadIdx.x;
        if (cell >= cells) continue;
        const bool k = known[t * cells + cell] != 0;
#pragma unroll
        for (int ch = 0; ch < 3; ch++) {
            const long long i = t * per + ch * cells + cell;
            vol[i] = k ? vals[i] : 0.0f;
        }
    }
}

// Page-locked host buffers for the inputs and results of host-buffer
// requests, kept per power-of-two size class and reused: copies between them
// and the device are asynchronous DMA, where pageable memory would make each
// copy a staged, synchronous one on the serving thread. The pool only grows
// (to the peak of buffers in use) and is freed with the server.
class PinnedPool {
   public:
    ~PinnedPool() {
        for (void* p : all_) cudaFreeHost(p);
    }
    void* get(size_t bytes, size_t& cap) {
        cap = kMin;
        while (cap < bytes) cap <<= 1;
        {
            std::lock_guard<std::mutex> g(mu_);
            auto& f = free_[cap];
            if (!f.empty()) {
                void* p = f.back();
                f.pop_back();
                return p;
            }
        }
        void* p = nullptr;
        cuda_check(cudaMallocHost(&p, cap), "cudaMallocHost", JC_OVER_BUDGET);
        std::lock_guard<std::mutex> g(mu_);
        all_.push_back(p);
        return p;
    }
    void put(void* p, size_t cap) {
        std::lock_guard<std::mutex> g(mu_);
        free_[cap].push_back(p);
    }

   private:
    static constexpr size_t kMin = 4096;
    std::mutex mu_;
    std::map<size_t, std::vector<void*>> free_;
    std::vector<void*> all_;
};

// A buffer of the pool, returned to it when the owner is destroyed or
// reassigned (move-only, like the request that owns it).
struct PinnedBuf {
    PinnedPool* pool = nullptr;
    void* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(PinnedPool& pl, size_t bytes) : pool(&pl) { p = pl.get(bytes, cap); }
    PinnedBuf(PinnedBuf&& o) noexcept : pool(o.pool), p(o.p), cap(o.cap) { o.p = nullptr; }
    PinnedBuf& operator=(PinnedBuf&& o) noexcept {
        if (this != &o) {
            reset();
            pool = o.pool;
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
        }
        return *this;
    }
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { reset(); }
    void reset() {
        if (p) pool->put(p, cap);
        p = nullptr;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

}  // namespace

// Request flag: x, known and meta are caller-owned device or page-locked host
// buffers (valid until the request is done), and so is jc_server_wait's `out`.
constexpr uint32_t kDeviceBuffers = JC_REQUEST_DEVICE_BUFFERS;

struct Request {
    uint64_t id = 0;
    jc_request r{};
    int status = JC_OK;
    std::string error;
    bool done = false, admitted = false, fresh = false;
    bool finished = false;  // set by the server thread; published as `done` under the lock
    bool device_io = false;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int ticks_done = 0;                  // forward / rewind
    int sweeps = 0, frozen = 0;          // reconstruct: host copy of the device bookkeeping
    float residual = 0.f;
    size_t cells = 0, bytes = 0;
    // page-locked copies of the inputs (host buffers), and the result
    PinnedBuf x, out, known, meta;
    // caller's device inputs (device buffers)
    const float* dev_x = nullptr;
    const uint8_t* dev_known = nullptr;
    const float* dev_meta = nullptr;
    // device buffers
    float* d_state = nullptr;   // forward / rewind: [3, cells]; reconstruct: the volume [H+1][3][cells]
    float* d_F = nullptr;       // reconstruct: [H][3][cells]
    float* d_R = nullptr;       // reconstruct: [H][3][cells]
    float* d_vals = nullptr;    // reconstruct: [H+1][3][cells]
    uint8_t* d_known = nullptr; // reconstruct: [H+1][cells]
    float* d_meta = nullptr;
    // staged at submit: its buffers reserved and its inputs copied on the
    // server's copy stream, complete when `ready` is
    bool reserved = false;
    cudaEvent_t ready = nullptr;
    ProjSlot* d_slot = nullptr;
    double energy = 0, max_viol = 0;
    bool recon() const { return r.task == JC_TASK_RECONSTRUCT; }
    long long inst_cells() const { return recon() ? 2 * (long long)r.ticks * (long long)cells : (long long)cells; }
    int n_inst() const { return recon() ? 2 * r.ticks : 2; }  // sub-instances; forward/rewind: init + tick
    int remaining() const { return recon() ? (frozen ? 0 : r.max_sweeps - sweeps) : r.ticks - ticks_done; }
    size_t out_floats() const { return (recon() ? (size_t)(r.ticks + 1) : 1) * 3 * cells; }
};

class Server {
   public:
    Server(jc_model* const* fwd, jc_model* const* rev, int n_grids, long long max_active_cells, double hbm_fraction);
    ~Server();
    uint64_t submit(const jc_request& r);
    void wait(uint64_t id, float* out, size_t out_len, jc_result* info, double timeout_s);
    void stats(jc_server_stats* s);
    void reset_stats();
    // Per-kernel device time (CUDA events around every launch of the loop):
    // start() clears and enables it, stop() disables it and returns
    // name -> (launches, total ms) of the iterations in between.
    void profile_start();
    std::map<std::string, std::pair<int, double>> profile_stop();

   private:
    PinnedPool pinned_;  // first member: outlives every request's buffers
    std::vector<Model*> fwd_, rev_;
    Dims dims_{};
    int precision_ = JC_FP32;
    DeviceArena arena_;
    Workspace ws_;
    cudaStream_t stream_ = nullptr;
    cudaStream_t wait_stream_ = nullptr;  // result copies of device-buffer requests in wait()
    cudaStream_t copy_stream_ = nullptr;  // inputs of requests staged at submit
    int unreserved_pending_ = 0;          // waiting requests without staged buffers
    InstDev* h_inst_ = nullptr;    // pinned mirror of the descriptor array
    CUtensorMap* h_maps_ = nullptr;  // pinned staging of the tensor maps (BF16), kMapsPerInst per instance
    ReconDev* h_recon_ = nullptr;  // pinned mirror of the reconstruct bookkeeping
    ReconDev* d_recon_ = nullptr;
    ProjSlot* h_slots_ = nullptr;  // pinned: slots of the requests finishing in a chunk
    int max_inst_ = 0, max_recon_ = 0;
    long long max_cells_ = 0;
    size_t budget_bytes_ = 0, used_bytes_ = 0;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<uint64_t> pending_;
    std::vector<uint64_t> active_;
    std::map<uint64_t, Request> reqs_;
    uint64_t next_id_ = 1;
    bool stop_ = false;
    std::thread thread_;
    // chunk timing: device events around each chunk, and the measured time
    // of one tick per active cell (for the chunk length when nothing waits)
    cudaEvent_t ev_first_ = nullptr, ev_a_ = nullptr, ev_b_ = nullptr;
    bool span_open_ = false;
    double s_per_cell_tick_ = 0.0;
    // statistics
    long long completed_ = 0;
    double cell_ticks_ = 0, busy_s_ = 0, first_submit_ = 0, last_done_ = 0, device_span_s_ = 0;
    int iterations_ = 0;
    long long launches_ = 0;
    bool profiling_ = false;
    std::map<std::string, std::pair<int, double>> prof_;

    void loop();
    int chunk_length(const std::vector<Request*>& act, long long head_cells, int head_inst) const;
    void iteration(std::vector<Request*>& act, int K);
    void admit_locked();
    void allocate(Request& q, cudaStream_t st);
    void release(Request& q);
    void release_on(Request& q, cudaStream_t st);
    void fail_locked(Request& q, int status, const std::string& msg);
};

Server::Server(jc_model* const* fwd, jc_model* const* rev, int n_grids, long long max_active_cells,
               double hbm_fraction) {
    if (!fwd || n_grids <= 0) throw Error(JC_BAD_ARGUMENT, "a server needs at least one forward model");
    if (max_active_cells <= 0) throw Error(JC_BAD_ARGUMENT, "max_active_cells must be > 0");
    if (!(hbm_fraction > 0.0 && hbm_fraction <= 1.0)) throw Error(JC_BAD_ARGUMENT, "hbm_fraction must be in (0, 1]");
    for (int i = 0; i < n_grids; i++) {
        if (!fwd[i]) throw Error(JC_BAD_ARGUMENT, "null forward model");
        fwd_.push_back(fwd[i]->m);
        if (rev) {
            if (!rev[i]) throw Error(JC_BAD_ARGUMENT, "null reverse model");
            rev_.push_back(rev[i]->m);
        }
    }
    dims_ = fwd_[0]->dims;
    precision_ = fwd_[0]->precision;
    auto check_family = [&](const std::vector<Model*>& ms) {
        for (Model* m : ms) {
            const Dims& d = m->dims;
            if (d.D != dims_.D || d.L != dims_.L || d.heads != dims_.heads || d.F != dims_.F || d.HD != dims_.HD ||
                d.P != dims_.P || d.mask_kind != dims_.mask_kind || d.radius != dims_.radius ||
                d.dilation != dims_.dilation || d.g != dims_.g || d.energy_r_max != dims_.energy_r_max ||
                d.norm_depth != dims_.norm_depth || m->precision != precision_)
                throw Error(JC_BAD_ARGUMENT, "the server's models must share hyper-parameters and precision");
            for (int k = 0; k < 3; k++)
                if (d.norm_mean[k] != dims_.norm_mean[k] || d.norm_std[k] != dims_.norm_std[k])
                    throw Error(JC_BAD_ARGUMENT, "the server's models must share the normalizer");
            if (m->w.shared_hash != ms[0]->w.shared_hash)
                throw Error(JC_BAD_ARGUMENT, "the models of one direction must share every tensor but pos");
        }
    };
    check_family(fwd_);
    if (!rev_.empty()) check_family(rev_);
    for (int i = 0; i < (int)rev_.size(); i++)
        if (rev_[i]->cfg.nx != fwd_[i]->cfg.nx || rev_[i]->cfg.ny != fwd_[i]->cfg.ny)
            throw Error(JC_BAD_ARGUMENT, "reverse model i must have forward model i's grid");
    max_cells_ = max_active_cells;
    max_inst_ = (int)std::min<long long>(max_active_cells / 16 + 64, 1 << 20);
    max_recon_ = max_inst_ / 2 + 1;
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaStreamCreateWithFlags(&wait_stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    for (cudaEvent_t* e : {&ev_first_, &ev_a_, &ev_b_}) cuda_check(cudaEventCreate(e), "cudaEventCreate");
    const int pp = dims_.P * dims_.P;
    ws_.alloc(arena_, dims_, (int)(max_cells_ / pp) + 1, max_cells_, max_inst_, fwd_[0]->w.bf16.get());
    d_recon_ = arena_.alloc_n<ReconDev>(max_recon_);
    cuda_check(cudaMallocHost(&h_inst_, (size_t)max_inst_ * sizeof(InstDev)), "cudaMallocHost", JC_OVER_BUDGET);
    if (precision_ == JC_BF16)
        cuda_check(cudaMallocHost(&h_maps_, (size_t)max_inst_ * kMapsPerInst * sizeof(CUtensorMap)), "cudaMallocHost",
                   JC_OVER_BUDGET);
    cuda_check(cudaMallocHost(&h_recon_, (size_t)max_recon_ * sizeof(ReconDev)), "cudaMallocHost", JC_OVER_BUDGET);
    cuda_check(cudaMallocHost(&h_slots_, (size_t)max_inst_ * sizeof(ProjSlot)), "cudaMallocHost", JC_OVER_BUDGET);
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    const double cap = hbm_fraction * (double)total_b - (double)(total_b - free_b);
    budget_bytes_ = cap > 0 ? (size_t)cap : 0;
    thread_ = std::thread([this] { loop(); });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    if (thread_.joinable()) thread_.join();
    for (auto& kv : reqs_) release(kv.second);
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
    if (wait_stream_) {
        cudaStreamSynchronize(wait_stream_);
        cudaStreamDestroy(wait_stream_);
    }
    if (copy_stream_) {
        cudaStreamSynchronize(copy_stream_);
        cudaStreamDestroy(copy_stream_);
    }
    for (cudaEvent_t e : {ev_first_, ev_a_, ev_b_})
        if (e) cudaEventDestroy(e);
    if (h_inst_) cudaFreeHost(h_inst_);
    if (h_maps_) cudaFreeHost(h_maps_);
    if (h_recon_) cudaFreeHost(h_recon_);
    if (h_slots_) cudaFreeHost(h_slots_);
}

uint64_t Server::submit(const jc_request& r) {
    if (r.grid < 0 || r.grid >= (int)fwd_.size()) throw Error(JC_BAD_ARGUMENT, "grid index out of range");
    if (r.task != JC_TASK_FORWARD && r.task != JC_TASK_REWIND && r.task != JC_TASK_RECONSTRUCT)
        throw Error(JC_BAD_ARGUMENT, "unknown task");
    if ((r.task != JC_TASK_FORWARD) && rev_.empty())
        throw Error(JC_BAD_ARGUMENT, "rewind and reconstruct need reverse models");
    if (r.ticks < 1) throw Error(JC_BAD_ARGUMENT, "ticks must be >= 1");
    if (r.flags & ~(3u | kDeviceBuffers)) throw Error(JC_BAD_ARGUMENT, "unknown request flag");
    if (!r.x || !r.meta) throw Error(JC_BAD_ARGUMENT, "null input");
    if (r.task == JC_TASK_RECONSTRUCT && (!r.known || r.max_sweeps < 1))
        throw Error(JC_BAD_ARGUMENT, "reconstruct needs a known mask and max_sweeps >= 1");
    const Model& m = *fwd_[r.grid];
    Request q;
    q.r = r;
    q.r.flags &= 3u;
    q.device_io = (r.flags & kDeviceBuffers) != 0;
    q.cells = (size_t)m.cfg.nx * m.cfg.ny;
    if (q.inst_cells() > max_cells_)
        throw Error(JC_OVER_BUDGET, "this request needs more cells per tick than the server's workspace holds");
    if (q.n_inst() > max_inst_)
        throw Error(JC_OVER_BUDGET, "this request needs more instances than the server's descriptor array holds");
    const size_t len = 3 * q.cells;
    if (r.task == JC_TASK_RECONSTRUCT) {
        const size_t vol = (size_t)(r.ticks + 1);
        if (q.device_io) {
            q.dev_x = r.x;
            q.dev_known = r.known;
        } else {
            q.x = PinnedBuf(pinned_, vol * len * 4);
            std::memcpy(q.x.p, r.x, vol * len * 4);
            q.known = PinnedBuf(pinned_, vol * q.cells);
            std::memcpy(q.known.p, r.known, vol * q.cells);
        }
        q.bytes = vol * len * 4 * 2 + 2 * (size_t)r.ticks * len * 4 + vol * q.cells + 4096;
    } else {
        if (q.device_io) q.dev_x = r.x;
        else {
            q.x = PinnedBuf(pinned_, len * 4);
            std::memcpy(q.x.p, r.x, len * 4);
        }
        q.bytes = len * 4 + 4096;
    }
    if (q.device_io) q.dev_meta = r.meta;
    else {
        q.meta = PinnedBuf(pinned_, (size_t)m.cfg.meta_dim * 4);
        std::memcpy(q.meta.p, r.meta, (size_t)m.cfg.meta_dim * 4);
    }
    q.r.x = nullptr;
    q.r.known = nullptr;
    q.r.meta = nullptr;
    if (q.bytes > budget_bytes_) throw Error(JC_OVER_BUDGET, "this request alone exceeds the device memory budget");
    // Stage now, while earlier chunks run: reserve the request's device
    // memory and copy its inputs on the copy stream, so that its admission
    // does not put those copies in front of the next chunk's kernels.
    // Only while no earlier request waits unstaged (memory is reserved in
    // arrival order) and the budget has room; else it is staged at admission.
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (unreserved_pending_ == 0 && used_bytes_ + q.bytes <= budget_bytes_) {
            used_bytes_ += q.bytes;
            q.reserved = true;
        }
    }
    long long staged_launches = 0;  // kernels launched here (reconstruct: the volume fill)
    if (q.reserved) {
        try {
            const long long l0 = g_launches;
            allocate(q, copy_stream_);
            staged_launches = g_launches - l0;
            cuda_check(cudaEventCreateWithFlags(&q.ready, cudaEventDisableTiming), "cudaEventCreate");
            cuda_check(cudaEventRecord(q.ready, copy_stream_), "cudaEventRecord");
        } catch (...) {
            release_on(q, copy_stream_);
            std::lock_guard<std::mutex> lk(mu_);
            used_bytes_ -= q.bytes;
            throw;
        }
    }
    std::lock_guard<std::mutex> lk(mu_);
    launches_ += staged_launches;
    if (!q.reserved) unreserved_pending_++;
    q.id = next_id_++;
    q.t_submit = now_s();
    if (first_submit_ == 0) first_submit_ = q.t_submit;
    const uint64_t id = q.id;
    reqs_.emplace(id, std::move(q));
    pending_.push_back(id);
    cv_work_.notify_one();
    return id;
}

void Server::wait(uint64_t id, float* out, size_t out_len, jc_result* info, double timeout_s) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = reqs_.find(id);
    if (it == reqs_.end()) throw Error(JC_NOT_FOUND, "unknown request id");
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (!it->second.done) {
        if (timeout_s >= 0 && cv_done_.wait_until(lk, deadline) == std::cv_status::timeout && !it->second.done)
            throw Error(JC_POLL, "timed out waiting for the request");
        if (timeout_s < 0) cv_done_.wait(lk);
        it = reqs_.find(id);
    }
    // a done request is no longer referenced by the server thread
    Request q = std::move(it->second);
    reqs_.erase(it);
    lk.unlock();
    if (q.status != JC_OK) throw Error((jc_status)q.status, q.error);
    const size_t n = q.out_floats();
    struct Settle {  // free the result's buffers and its budget, even on errors
        Server* s;
        Request* q;
        ~Settle() {
            s->release_on(*q, s->wait_stream_);
            cudaStreamSynchronize(s->wait_stream_);
            {
                std::lock_guard<std::mutex> g(s->mu_);
                s->used_bytes_ -= q->bytes;
            }
            s->cv_work_.notify_one();  // the freed memory may admit a waiting request
        }
    } settle{this, &q};
    if (out && out_len < n) throw Error(JC_BAD_ARGUMENT, "output buffer too small");
    if (q.device_io) {
        // the result is in the request's device buffer, written by work that
        // has completed (the chunk that finished it was synchronized)
        if (out) {
            cuda_check(cudaMemcpyAsync(out, q.d_state, n * 4, cudaMemcpyDefault, wait_stream_), "result copy", JC_MAP);
            cuda_check(cudaStreamSynchronize(wait_stream_), "cudaStreamSynchronize", JC_POLL);
        }
    } else if (out) {
        // host result: device -> the server's page-locked staging buffer -> `out`
        q.out = PinnedBuf(pinned_, n * 4);
        cuda_check(cudaMemcpyAsync(q.out.p, q.d_state, n * 4, cudaMemcpyDeviceToHost, wait_stream_), "D2H", JC_MAP);
        cuda_check(cudaStreamSynchronize(wait_stream_), "cudaStreamSynchronize", JC_POLL);
        std::memcpy(out, q.out.p, n * 4);
    }
    if (info) {
        info->latency_s = q.t_done - q.t_submit;
        info->queue_s = q.t_admit - q.t_submit;
        info->sweeps = q.sweeps;
        info->residual = q.residual;
        info->energy = q.energy;
        info->max_violation = q.max_viol;
        info->out_len = (int64_t)n;
    }
}

void Server::stats(jc_server_stats* s) {
    std::lock_guard<std::mutex> lk(mu_);
    s->completed = completed_;
    s->cell_ticks = cell_ticks_;
    s->busy_s = busy_s_;
    s->span_s = last_done_ > first_submit_ ? last_done_ - first_submit_ : 0.0;
    s->iterations = iterations_;
    s->active = (int32_t)active_.size();
    s->pending = (int32_t)pending_.size();
    s->device_span_s = device_span_s_;
    s->launches = launches_;
}

void Server::reset_stats() {
    std::lock_guard<std::mutex> lk(mu_);
    completed_ = 0;
    cell_ticks_ = busy_s_ = device_span_s_ = 0.0;
    first_submit_ = last_done_ = 0.0;
    iterations_ = 0;
    launches_ = 0;
    span_open_ = false;
}

void Server::profile_start() {
    std::lock_guard<std::mutex> lk(mu_);
    prof_.clear();
    profiling_ = true;
}

std::map<std::string, std::pair<int, double>> Server::profile_stop() {
    std::lock_guard<std::mutex> lk(mu_);
    profiling_ = false;
    std::map<std::string, std::pair<int, double>> out;
    out.swap(prof_);
    return out;
}

void Server::fail_locked(Request& q, int status, const std::string& msg) {
    q.status = status;
    q.error = msg;
    q.done = true;
    q.t_done = now_s();
}

void Server::allocate(Request& q, cudaStream_t st) {
    const size_t len = 3 * q.cells;
    auto get = [&](size_t bytes) {
        void* p = nullptr;
        cuda_check(cudaMallocAsync(&p, bytes, st), "cudaMallocAsync", JC_OVER_BUDGET);
        return p;
    };
    // caller-owned buffers: device or page-locked host memory (unified addressing tells which)
    const cudaMemcpyKind in_kind = q.device_io ? cudaMemcpyDefault : cudaMemcpyHostToDevice;
    q.d_meta = static_cast<float*>(get(64 * 4));
    q.d_slot = static_cast<ProjSlot*>(get(sizeof(ProjSlot)));
    cuda_check(cudaMemcpyAsync(q.d_meta, q.device_io ? q.dev_meta : q.meta.as<float>(), dims_.meta_dim * 4, in_kind,
                               st),
               "meta", JC_MAP);
    if (q.recon()) {
        const size_t H = (size_t)q.r.ticks;
        q.d_state = static_cast<float*>(get((H + 1) * len * 4));
        q.d_vals = static_cast<float*>(get((H + 1) * len * 4));
        q.d_F = static_cast<float*>(get(H * len * 4));
        q.d_R = static_cast<float*>(get(H * len * 4));
        q.d_known = static_cast<uint8_t*>(get((H + 1) * q.cells));
        cuda_check(cudaMemcpyAsync(q.d_vals, q.device_io ? q.dev_x : q.x.as<float>(), (H + 1) * len * 4, in_kind, st),
                   "reconstruct values", JC_MAP);
        cuda_check(cudaMemcpyAsync(q.d_known, q.device_io ? q.dev_known : q.known.as<uint8_t>(), (H + 1) * q.cells, in_kind,
                                   st),
                   "reconstruct mask", JC_MAP);
        KScope k("recon_fill", st);
        recon_fill_kernel<<<(unsigned)std::min<size_t>((H + 1) * ((q.cells + 255) / 256), 4096), 256, 0, st>>>(
            q.d_state, q.d_vals, q.d_known, (int)H, (long long)q.cells);
        cuda_check(cudaGetLastError(), "reconstruct fill");
    } else {
        q.d_state = static_cast<float*>(get(len * 4));
        cuda_check(cudaMemcpyAsync(q.d_state, q.device_io ? q.dev_x : q.x.as<float>(), len * 4, in_kind, st), "state",
                   JC_MAP);
    }
}

void Server::release(Request& q) { release_on(q, stream_); }

void Server::release_on(Request& q, cudaStream_t st) {
    // buffers staged at submit: the frees follow the staging copies
    if (q.ready) cudaStreamWaitEvent(st, q.ready, 0);
    for (void* p : {(void*)q.d_state, (void*)q.d_F, (void*)q.d_R, (void*)q.d_vals, (void*)q.d_known,
                    (void*)q.d_meta, (void*)q.d_slot})
        if (p) cudaFreeAsync(p, st);
    if (q.ready) cudaEventDestroy(q.ready);
    q.ready = nullptr;
    q.d_state = q.d_F = q.d_R = q.d_vals = nullptr;
    q.d_known = nullptr;
    q.d_meta = nullptr;
    q.d_slot = nullptr;
}

void Server::admit_locked() {
    long long cells = 0;
    int inst = 0;
    for (uint64_t id : active_) {
        const Request& q = reqs_[id];
        cells += q.inst_cells();
        inst += q.n_inst();
    }
    while (!pending_.empty()) {
        Request& q = reqs_[pending_.front()];
        if (cells + q.inst_cells() > max_cells_ || inst + q.n_inst() > max_inst_ ||
            (!q.reserved && used_bytes_ + q.bytes > budget_bytes_))
            break;  // first in, first admitted: later requests wait behind it
        pending_.pop_front();
        cells += q.inst_cells();
        inst += q.n_inst();
        if (!q.reserved) {
            used_bytes_ += q.bytes;
            unreserved_pending_--;
        }
        q.admitted = true;
        q.fresh = true;
        q.t_admit = now_s();
        active_.push_back(q.id);
    }
}

// Ticks of the next chunk. Nothing waits: the longest remaining request, at
// most about kChunkTargetS of device time (measured per active cell-tick).
// A request waits for room: up to the first tick after which enough of the
// active requests have finished to admit it.
int Server::chunk_length(const std::vector<Request*>& act, long long head_cells, int head_inst) const {
    int most = 1;
    long long cells = 0;
    int inst = 0;
    std::vector<std::pair<int, Request*>> ends;
    for (Request* q : act) {
        const int rem = q->remaining();
        most = std::max(most, rem);
        cells += q->inst_cells();
        inst += q->n_inst();
        ends.push_back({rem, q});
    }
    int K = std::min(most, kMaxChunk);
    if (head_cells < 0) {
        if (s_per_cell_tick_ > 0.0 && cells > 0) {
            const double tick_s = s_per_cell_tick_ * (double)cells;
            K = std::min(K, std::max(1, (int)(kChunkTargetS / tick_s)));
        }
        return K;
    }
    std::sort(ends.begin(), ends.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    for (const auto& e : ends) {
        cells -= e.second->inst_cells();
        inst -= e.second->n_inst();
        if (cells + head_cells <= max_cells_ && inst + head_inst <= max_inst_) return std::max(1, std::min(K, e.first));
    }
    return K;
}

void Server::loop() {
    std::vector<Request*> act;
    KernelTimer kt;
    while (true) {
        long long head_cells = -1;
        int head_inst = 0;
        bool prof = false;
        {
            std::unique_lock<std::mutex> lk(mu_);
            admit_locked();
            while (active_.empty() && !stop_) {
                cv_work_.wait(lk);
                admit_locked();
            }
            if (stop_) return;
            act.clear();
            for (uint64_t id : active_) act.push_back(&reqs_[id]);
            if (!pending_.empty()) {
                const Request& h = reqs_[pending_.front()];
                head_cells = h.inst_cells();
                head_inst = h.n_inst();
            }
            prof = profiling_;
        }
        const int K = chunk_length(act, head_cells, head_inst);
        const double t0 = now_s();
        const long long l0 = g_launches;
        if (prof) g_ktimer = &kt;
        try {
            iteration(act, K);
            if (prof) {
                g_ktimer = nullptr;
                auto sm = kt.summary();
                std::lock_guard<std::mutex> lk(mu_);
                for (const auto& kv : sm) {
                    auto& v = prof_[kv.first];
                    v.first += kv.second.first;
                    v.second += kv.second.second;
                }
            }
        } catch (const std::exception& e) {
            g_ktimer = nullptr;
            kt.summary();
            const Error* je = dynamic_cast<const Error*>(&e);
            cudaStreamSynchronize(stream_);
            cudaGetLastError();
            std::lock_guard<std::mutex> lk(mu_);
            for (Request* q : act) {
                release(*q);
                used_bytes_ -= q->bytes;
                fail_locked(*q, je ? je->code : JC_CUDA_ERROR, e.what());
            }
            active_.clear();
            span_open_ = false;
            cv_done_.notify_all();
            continue;
        }
        std::lock_guard<std::mutex> lk(mu_);
        busy_s_ += now_s() - t0;
        iterations_++;
        launches_ += g_launches - l0;
        std::vector<uint64_t> still;
        for (Request* q : act) {
            if (q->finished) {
                q->done = true;
                completed_++;
                cell_ticks_ += (double)q->cells * q->r.ticks;
                last_done_ = q->t_done;
                // the result's memory is freed (and its budget returned) in wait()
            } else {
                still.push_back(q->id);
            }
        }
        active_.swap(still);
        cv_done_.notify_all();
    }
}

namespace {

// The instances of one weight group in a chunk, ordered by the ticks their
// request has left (longest first), with cumulative sizes so that the
// instances still running at chunk tick t form a prefix view.
struct GroupPlan {
    std::vector<InstDev> inst;
    std::vector<int> rem;  // per instance: ticks (sweeps) its request has left
    std::vector<int> rows, tiles, ttiles, ctiles;
    std::vector<long long> cells, maxc;
    int inst_base = 0, row_base = 0;
    long long cell_base = 0;
    void add(InstDev d, int r) {
        const int r0 = rows.empty() ? 0 : rows.back();
        const long long c0 = cells.empty() ? 0 : cells.back();
        const int t0 = tiles.empty() ? 0 : tiles.back(), tt0 = ttiles.empty() ? 0 : ttiles.back(),
                  ct0 = ctiles.empty() ? 0 : ctiles.back();
        d.row0 = r0;
        d.cell0 = c0;
        d.tile0 = t0;
        d.tt0 = tt0;
        d.ct0 = ct0;
        inst.push_back(d);
        rem.push_back(r);
        rows.push_back(r0 + d.tx * d.ty);
        cells.push_back(c0 + (long long)d.nx * d.ny);
        tiles.push_back(t0 + cell_tiles(d.nx, d.ny));
        ttiles.push_back(tt0 + conv_tiles(d.tx, d.ty));
        ctiles.push_back(ct0 + conv_tiles(d.nx, d.ny));
        maxc.push_back(std::max(maxc.empty() ? 0LL : maxc.back(), (long long)d.nx * d.ny));
    }
    // instances still running at chunk tick t (rem >= t)
    int running(int t) const {
        int n = 0;
        while (n < (int)rem.size() && rem[n] >= t) n++;
        return n;
    }
    Pack view(const Workspace& ws, const Dims& d, int n) const {
        Pack v = ws.view(d, inst_base, n, row_base, rows[n - 1], cell_base, cells[n - 1], tiles[n - 1],
                         ttiles[n - 1], ctiles[n - 1]);
        v.max_inst_cells = maxc[n - 1];
        return v;
    }
};

}  // namespace

void Server::iteration(std::vector<Request*>& act, int K) {
    cudaStream_t s = stream_;
    // new requests: buffers and inputs on the device
    for (Request* q : act) {
        if (!q->fresh) continue;
        if (q->ready) cuda_check(cudaStreamWaitEvent(s, q->ready, 0), "cudaStreamWaitEvent");  // staged at submit
        else if (!q->d_state) allocate(*q, s);
    }
    auto base_inst = [&](const Model& m) {
        InstDev d{};
        d.tx = m.cfg.nx / m.cfg.patch;
        d.ty = m.cfg.ny / m.cfg.patch;
        d.nx = m.cfg.nx;
        d.ny = m.cfg.ny;
        d.pos = m.w.pos;
        return d;
    };
    // requests of each group, longest remaining first (stable: admission order)
    std::vector<Request*> order(act.begin(), act.end());
    std::stable_sort(order.begin(), order.end(),
                     [](const Request* a, const Request* b) { return a->remaining() > b->remaining(); });
    std::vector<InstDev> init, proj;
    std::vector<int> proj_rem;
    std::vector<long long> proj_maxc;
    GroupPlan fg, rg;
    std::vector<Request*> recon;
    for (Request* q : order) {
        const int g = q->r.grid, rem = q->remaining();
        if (q->recon()) {
            if (rem <= 0) continue;
            const size_t len = 3 * q->cells;
            for (int t = 1; t <= q->r.ticks; t++) {  // F_t = step_F(X_{t-1})
                InstDev d = base_inst(*fwd_[g]);
                d.state = q->d_state + (size_t)(t - 1) * len;
                d.out = q->d_F + (size_t)(t - 1) * len;
                d.meta = q->d_meta;
                d.flags = 4u;
                fg.add(d, rem);
            }
            for (int t = 0; t < q->r.ticks; t++) {  // R_t = step_R(X_{t+1})
                InstDev d = base_inst(*rev_[g]);
                d.state = q->d_state + (size_t)(t + 1) * len;
                d.out = q->d_R + (size_t)t * len;
                d.meta = q->d_meta;
                d.flags = 4u;
                rg.add(d, rem);
            }
            recon.push_back(q);
        } else {
            const Model& m = q->r.task == JC_TASK_FORWARD ? *fwd_[g] : *rev_[g];
            InstDev d = base_inst(m);
            d.state = q->d_state;
            d.out = q->d_state;
            d.meta = q->d_meta;
            d.flags = q->r.flags;
            d.slot = q->d_slot;
            if (q->fresh) init.push_back(d);
            (q->r.task == JC_TASK_FORWARD ? fg : rg).add(d, rem);
            proj.push_back(d);
            proj_rem.push_back(rem);
            proj_maxc.push_back(std::max(proj_maxc.empty() ? 0LL : proj_maxc.back(), (long long)d.nx * d.ny));
        }
    }
    // descriptor array: [init projections] [forward group] [reverse group]
    // [tick projections: forward and rewind requests, longest remaining first]
    fg.inst_base = (int)init.size();
    rg.inst_base = fg.inst_base + (int)fg.inst.size();
    rg.row_base = fg.rows.empty() ? 0 : fg.rows.back();
    rg.cell_base = fg.cells.empty() ? 0 : fg.cells.back();
    const int proj_base = rg.inst_base + (int)rg.inst.size();
    const int n_all = proj_base + (int)proj.size();
    if (n_all > max_inst_) throw Error(JC_OVER_BUDGET, "too many instances for the server's descriptor array");
    if ((long long)rg.row_base + (rg.rows.empty() ? 0 : rg.rows.back()) > ws_.max_rows ||
        rg.cell_base + (rg.cells.empty() ? 0 : rg.cells.back()) > ws_.max_cells)
        throw Error(JC_OVER_BUDGET, "the active requests need more cells than the server's workspace holds");
    std::memcpy(h_inst_, init.data(), init.size() * sizeof(InstDev));
    std::memcpy(h_inst_ + fg.inst_base, fg.inst.data(), fg.inst.size() * sizeof(InstDev));
    std::memcpy(h_inst_ + rg.inst_base, rg.inst.data(), rg.inst.size() * sizeof(InstDev));
    std::memcpy(h_inst_ + proj_base, proj.data(), proj.size() * sizeof(InstDev));
    cuda_check(cudaMemcpyAsync(ws_.base.inst, h_inst_, (size_t)n_all * sizeof(InstDev), cudaMemcpyHostToDevice, s),
               "descriptors", JC_MAP);
    // reconstruct bookkeeping, in the same (longest remaining first) order
    for (size_t i = 0; i < recon.size(); i++) {
        const Request* q = recon[i];
        ReconDev& R = h_recon_[i];
        R = ReconDev{};
        R.vol = q->d_state;
        R.F = q->d_F;
        R.R = q->d_R;
        R.vals = q->d_vals;
        R.known = q->d_known;
        R.cells = (long long)q->cells;
        R.H = q->r.ticks;
        R.max_sweeps = q->r.max_sweeps;
        R.tol = q->r.tol;
        R.sweeps = q->sweeps;
        R.frozen = q->frozen;
        R.last_resid = q->residual;
    }
    if (!recon.empty())
        cuda_check(cudaMemcpyAsync(d_recon_, h_recon_, recon.size() * sizeof(ReconDev), cudaMemcpyHostToDevice, s),
                   "reconstruct bookkeeping", JC_MAP);
    const BF16Path* bf = fwd_[0]->w.bf16.get();
    if (bf) {
        if (!fg.inst.empty()) {
            Pack v = fg.view(ws_, dims_, (int)fg.inst.size());
            bf->prepare(dims_, v, h_inst_ + fg.inst_base, s, h_maps_ + (size_t)fg.inst_base * kMapsPerInst);
            bf->tune(dims_, fwd_[0]->w.f32, v, s);
        }
        if (!rg.inst.empty()) {
            Pack v = rg.view(ws_, dims_, (int)rg.inst.size());
            bf->prepare(dims_, v, h_inst_ + rg.inst_base, s, h_maps_ + (size_t)rg.inst_base * kMapsPerInst);
            rev_[0]->w.bf16->tune(dims_, rev_[0]->w.f32, v, s);
        }
    }
    // the chunk: K ticks with no host round trip
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (!span_open_) {
            cuda_check(cudaEventRecord(ev_first_, s), "cudaEventRecord");
            span_open_ = true;
        }
    }
    cuda_check(cudaEventRecord(ev_a_, s), "cudaEventRecord");
    long long cell_ticks = 0;
    for (int t = 1; t <= K; t++) {
        if (t == 1 && !init.empty()) {
            Pack pi = ws_.view(dims_, 0, (int)init.size(), 0, 0, 0, 0, 0, 0, 0);
            long long mx = 0;
            for (const InstDev& d : init) mx = std::max(mx, (long long)d.nx * d.ny);
            pi.max_inst_cells = mx;
            projection(dims_, pi, 1, s);
        }
        const int nf = fg.running(t), nr = rg.running(t);
        if (nf) {
            Pack v = fg.view(ws_, dims_, nf);
            fwd_[0]->forward_pack(v, kWriteNextState, s);
            cell_ticks += v.NC;
        }
        if (nr) {
            Pack v = rg.view(ws_, dims_, nr);
            rev_[0]->forward_pack(v, kWriteNextState, s);
            cell_ticks += v.NC;
        }
        int np = 0;
        while (np < (int)proj.size() && proj_rem[np] >= t) np++;
        if (np) {
            Pack pv = ws_.view(dims_, proj_base, np, 0, 0, 0, 0, 0, 0, 0);
            pv.max_inst_cells = proj_maxc[np - 1];
            projection(dims_, pv, 0, s);
        }
        int nrec = 0;
        long long rc = 0;
        int rh = 0;
        while (nrec < (int)recon.size() && recon[nrec]->remaining() >= t) {
            rc = std::max(rc, (long long)recon[nrec]->cells);
            rh = std::max(rh, recon[nrec]->r.ticks);
            nrec++;
        }
        if (nrec) {
            recon_update(d_recon_, nrec, rc, rh, s);
            recon_finalize(d_recon_, nrec, 0ull, 0, s);
        }
    }
    cuda_check(cudaEventRecord(ev_b_, s), "cudaEventRecord");
    // results of forward/rewind requests that finish in this chunk
    std::vector<Request*> finishing;
    for (Request* q : act) {
        if (q->recon() || q->remaining() > K) continue;
        cuda_check(cudaMemcpyAsync(&h_slots_[finishing.size()], q->d_slot, sizeof(ProjSlot), cudaMemcpyDeviceToHost, s),
                   "D2H", JC_MAP);
        finishing.push_back(q);
    }
    if (!recon.empty())
        cuda_check(cudaMemcpyAsync(h_recon_, d_recon_, recon.size() * sizeof(ReconDev), cudaMemcpyDeviceToHost, s),
                   "D2H", JC_MAP);
    cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    ws_.check_timeout(s);
    {
        float ms = 0.f, span = 0.f;
        cudaEventElapsedTime(&ms, ev_a_, ev_b_);
        cudaEventElapsedTime(&span, ev_first_, ev_b_);
        if (cell_ticks > 0 && ms > 0.f) {
            const double v = ms * 1e-3 / (double)cell_ticks;
            s_per_cell_tick_ = s_per_cell_tick_ > 0.0 ? 0.5 * (s_per_cell_tick_ + v) : v;
        }
        std::lock_guard<std::mutex> lk(mu_);
        device_span_s_ = span * 1e-3;
    }
    const double t = now_s();
    for (size_t i = 0; i < finishing.size(); i++) {
        Request* q = finishing[i];
        q->energy = h_slots_[i].energy;
        q->max_viol = h_slots_[i].max_viol;
    }
    for (Request* q : act) {
        if (q->fresh) {  // its inputs are on the device (the chunk above waited for them): back to the pool
            q->x.reset();
            q->known.reset();
            q->meta.reset();
        }
        q->fresh = false;
        if (q->recon()) continue;
        const int rem = q->remaining();
        q->ticks_done += std::min(rem, K);
        if (q->ticks_done == q->r.ticks) {  // the result stays on the device until wait()
            q->finished = true;
            q->t_done = t;
        }
    }
    std::vector<Request*> recon_done;
    for (size_t i = 0; i < recon.size(); i++) {
        Request* q = recon[i];
        q->sweeps = h_recon_[i].sweeps;
        q->frozen = h_recon_[i].frozen;
        q->residual = h_recon_[i].last_resid;
        if (q->frozen) recon_done.push_back(q);
    }
    for (Request* q : recon_done) {  // the volume stays on the device until wait()
        q->finished = true;
        q->t_done = t;
    }
}

}  // namespace jc

struct jc_server {
    jc::Server* s;
};

namespace jc {
jc_status server_create(jc_model* const* fwd, jc_model* const* rev, int32_t n, int64_t max_cells, double frac,
                        jc_server** out) {
    *out = new jc_server{new Server(fwd, rev, n, max_cells, frac)};
    return JC_OK;
}
void server_destroy(jc_server* s) {
    delete s->s;
    delete s;
}
uint64_t server_submit(jc_server* s, const jc_request* r) { return s->s->submit(*r); }
void server_wait(jc_server* s, uint64_t id, float* out, size_t n, jc_result* info, double timeout) {
    s->s->wait(id, out, n, info, timeout);
}
void server_stats(jc_server* s, jc_server_stats* st) { s->s->stats(st); }
void server_reset_stats(jc_server* s) { s->s->reset_stats(); }
void server_profile(jc_server* s, int enable, char* report, size_t cap) {
    if (enable) {
        s->s->profile_start();
        return;
    }
    const auto m = s->s->profile_stop();
    if (!report || cap == 0) return;
    std::string out;
    for (const auto& kv : m)
        out += kv.first + "," + std::to_string(kv.second.first) + "," + std::to_string(kv.second.second) + "\n";
    const size_t n = std::min(out.size(), cap - 1);
    std::memcpy(report, out.data(), n);
    report[n] = 0;
}
}  // namespace jc
