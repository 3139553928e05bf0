// Serving loop: continuous batching of forward, rewind and reconstruct
// requests of different grid sizes on one GPU.
//
// A server thread runs iterations; each iteration is one tick for every active
// request. All instances that use the forward weights go into one packed launch
// sequence, all that use the reverse weights into another:
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
// Requests that arrive while others run are admitted at the next iteration,
// while their instances fit the workspace and their buffers fit the device
// memory budget; each request's state stays on the device until it is done.
// A request's result does not depend on which other requests share its
// launches (no kernel's arithmetic for one instance reads another's data).
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

// X_t <- known_t ? value : mean of the available step results; records the
// largest change of an unknown value (as the bits of a non-negative float).
__global__ void recon_update_kernel(float* __restrict__ vol, const float* __restrict__ F,
                                    const float* __restrict__ Rv, const float* __restrict__ vals,
                                    const uint8_t* __restrict__ known, int H, long long cells,
                                    unsigned* __restrict__ residual) {
    __shared__ float red[32];
    const long long per = 3 * cells, total = (long long)(H + 1) * per;
    float local = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / per);
        const long long rem = i - (long long)t * per, cell = rem % cells;
        float v;
        if (known[(long long)t * cells + cell]) {
            v = vals[i];
        } else {
            if (t == 0) v = Rv[rem];
            else if (t == H) v = F[(long long)(H - 1) * per + rem];
            else v = 0.5f * (F[(long long)(t - 1) * per + rem] + Rv[(long long)t * per + rem]);
            local = fmaxf(local, fabsf(v - vol[i]));
        }
        vol[i] = v;
    }
    local = warp_max(local);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        v = warp_max(v);
        if (threadIdx.x == 0) atomicMax(residual, __float_as_uint(v));
    }
}

// X_t <- known_t ? value : 0 (the normalized mean state) for every t.
__global__ void recon_init_kernel(float* __restrict__ vol, const float* __restrict__ vals,
                                  const uint8_t* __restrict__ known, int H, long long cells) {
    const long long per = 3 * cells, total = (long long)(H + 1) * per;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / per);
        const long long cell = (i - (long long)t * per) % cells;
        vol[i] = known[(long long)t * cells + cell] ? vals[i] : 0.0f;
    }
}

}  // namespace

struct Request {
    uint64_t id = 0;
    jc_request r{};
    int status = JC_OK;
    std::string error;
    bool done = false, admitted = false, fresh = false;
    bool finished = false;  // set by the server thread; published as `done` under the lock
    double t_submit = 0, t_admit = 0, t_done = 0;
    int ticks_done = 0, sweeps = 0;
    float residual = 0.f;
    size_t cells = 0, bytes = 0;
    // host copies of the inputs, and the result
    std::vector<float> x, out;
    std::vector<uint8_t> known;
    std::vector<float> meta;
    // device buffers
    float* d_state = nullptr;   // forward / rewind: [3, cells]; reconstruct: the volume [H+1][3][cells]
    float* d_F = nullptr;       // reconstruct: [H][3][cells]
    float* d_R = nullptr;       // reconstruct: [H][3][cells]
    float* d_vals = nullptr;    // reconstruct: [H+1][3][cells]
    uint8_t* d_known = nullptr; // reconstruct: [H+1][cells]
    float* d_meta = nullptr;
    ProjSlot* d_slot = nullptr;
    unsigned* d_resid = nullptr;
    double energy = 0, max_viol = 0;
    int inst_cells() const {
        return r.task == JC_TASK_RECONSTRUCT ? (int)(2 * (size_t)r.ticks * cells) : (int)cells;
    }
};

class Server {
   public:
    Server(jc_model* const* fwd, jc_model* const* rev, int n_grids, long long max_active_cells, double hbm_fraction);
    ~Server();
    uint64_t submit(const jc_request& r);
    void wait(uint64_t id, float* out, size_t out_len, jc_result* info, double timeout_s);
    void stats(jc_server_stats* s);

   private:
    std::vector<Model*> fwd_, rev_;
    Dims dims_{};
    int precision_ = JC_FP32;
    DeviceArena arena_;
    Workspace ws_;
    cudaStream_t stream_ = nullptr;
    InstDev* h_inst_ = nullptr;  // pinned mirror of the descriptor array
    int max_inst_ = 0;
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
    // statistics
    long long completed_ = 0;
    double cell_ticks_ = 0, busy_s_ = 0, first_submit_ = 0, last_done_ = 0;
    int iterations_ = 0;

    void loop();
    void iteration(std::vector<Request*>& act);
    void admit_locked();
    void allocate(Request& q);
    void release(Request& q);
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
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    const int pp = dims_.P * dims_.P;
    ws_.alloc(arena_, dims_, (int)(max_cells_ / pp) + 1, max_cells_, max_inst_, fwd_[0]->w.bf16.get());
    cuda_check(cudaMallocHost(&h_inst_, (size_t)max_inst_ * sizeof(InstDev)), "cudaMallocHost", JC_OVER_BUDGET);
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
    if (h_inst_) cudaFreeHost(h_inst_);
}

uint64_t Server::submit(const jc_request& r) {
    if (r.grid < 0 || r.grid >= (int)fwd_.size()) throw Error(JC_BAD_ARGUMENT, "grid index out of range");
    if (r.task != JC_TASK_FORWARD && r.task != JC_TASK_REWIND && r.task != JC_TASK_RECONSTRUCT)
        throw Error(JC_BAD_ARGUMENT, "unknown task");
    if ((r.task != JC_TASK_FORWARD) && rev_.empty())
        throw Error(JC_BAD_ARGUMENT, "rewind and reconstruct need reverse models");
    if (r.ticks < 1) throw Error(JC_BAD_ARGUMENT, "ticks must be >= 1");
    if (r.flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown projection flag");
    if (!r.x || !r.meta) throw Error(JC_BAD_ARGUMENT, "null input");
    if (r.task == JC_TASK_RECONSTRUCT && (!r.known || r.max_sweeps < 1))
        throw Error(JC_BAD_ARGUMENT, "reconstruct needs a known mask and max_sweeps >= 1");
    const Model& m = *fwd_[r.grid];
    Request q;
    q.r = r;
    q.cells = (size_t)m.cfg.nx * m.cfg.ny;
    if (q.inst_cells() > max_cells_)
        throw Error(JC_OVER_BUDGET, "this request needs more cells per tick than the server's workspace holds");
    const size_t len = 3 * q.cells;
    if (r.task == JC_TASK_RECONSTRUCT) {
        const size_t vol = (size_t)(r.ticks + 1);
        q.x.assign(r.x, r.x + vol * len);
        q.known.assign(r.known, r.known + vol * q.cells);
        q.bytes = vol * len * 4 * 2 + 2 * (size_t)r.ticks * len * 4 + vol * q.cells + 4096;
    } else {
        q.x.assign(r.x, r.x + len);
        q.bytes = len * 4 + 4096;
    }
    q.meta.assign(r.meta, r.meta + m.cfg.meta_dim);
    q.r.x = nullptr;
    q.r.known = nullptr;
    q.r.meta = nullptr;
    if (q.bytes > budget_bytes_) throw Error(JC_OVER_BUDGET, "this request alone exceeds the device memory budget");
    std::lock_guard<std::mutex> lk(mu_);
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
    Request& q = it->second;
    if (q.status != JC_OK) {
        Error e((jc_status)q.status, q.error);
        reqs_.erase(it);
        throw e;
    }
    if (out) {
        if (out_len < q.out.size()) throw Error(JC_BAD_ARGUMENT, "output buffer too small");
        std::memcpy(out, q.out.data(), q.out.size() * 4);
    }
    if (info) {
        info->latency_s = q.t_done - q.t_submit;
        info->queue_s = q.t_admit - q.t_submit;
        info->sweeps = q.sweeps;
        info->residual = q.residual;
        info->energy = q.energy;
        info->max_violation = q.max_viol;
        info->out_len = (int64_t)q.out.size();
    }
    reqs_.erase(it);
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
}

void Server::fail_locked(Request& q, int status, const std::string& msg) {
    q.status = status;
    q.error = msg;
    q.done = true;
    q.t_done = now_s();
}

void Server::allocate(Request& q) {
    const size_t len = 3 * q.cells;
    auto get = [&](size_t bytes) {
        void* p = nullptr;
        cuda_check(cudaMallocAsync(&p, bytes, stream_), "cudaMallocAsync", JC_OVER_BUDGET);
        return p;
    };
    q.d_meta = static_cast<float*>(get(64 * 4));
    q.d_slot = static_cast<ProjSlot*>(get(sizeof(ProjSlot)));
    q.d_resid = static_cast<unsigned*>(get(16));
    cuda_check(cudaMemcpyAsync(q.d_meta, q.meta.data(), q.meta.size() * 4, cudaMemcpyHostToDevice, stream_), "H2D",
               JC_MAP);
    if (q.r.task == JC_TASK_RECONSTRUCT) {
        const size_t H = (size_t)q.r.ticks;
        q.d_state = static_cast<float*>(get((H + 1) * len * 4));
        q.d_vals = static_cast<float*>(get((H + 1) * len * 4));
        q.d_F = static_cast<float*>(get(H * len * 4));
        q.d_R = static_cast<float*>(get(H * len * 4));
        q.d_known = static_cast<uint8_t*>(get((H + 1) * q.cells));
        cuda_check(cudaMemcpyAsync(q.d_vals, q.x.data(), (H + 1) * len * 4, cudaMemcpyHostToDevice, stream_), "H2D",
                   JC_MAP);
        cuda_check(cudaMemcpyAsync(q.d_known, q.known.data(), (H + 1) * q.cells, cudaMemcpyHostToDevice, stream_),
                   "H2D", JC_MAP);
        recon_init_kernel<<<1024, 256, 0, stream_>>>(q.d_state, q.d_vals, q.d_known, (int)H, (long long)q.cells);
        cuda_check(cudaGetLastError(), "recon init");
    } else {
        q.d_state = static_cast<float*>(get(len * 4));
        cuda_check(cudaMemcpyAsync(q.d_state, q.x.data(), len * 4, cudaMemcpyHostToDevice, stream_), "H2D", JC_MAP);
    }
}

void Server::release(Request& q) {
    for (void* p : {(void*)q.d_state, (void*)q.d_F, (void*)q.d_R, (void*)q.d_vals, (void*)q.d_known,
                    (void*)q.d_meta, (void*)q.d_slot, (void*)q.d_resid})
        if (p) cudaFreeAsync(p, stream_);
    q.d_state = q.d_F = q.d_R = q.d_vals = nullptr;
    q.d_known = nullptr;
    q.d_meta = nullptr;
    q.d_slot = nullptr;
    q.d_resid = nullptr;
}

void Server::admit_locked() {
    long long cells = 0;
    for (uint64_t id : active_) cells += reqs_[id].inst_cells();
    int inst = 0;
    for (uint64_t id : active_) {
        const Request& q = reqs_[id];
        inst += q.r.task == JC_TASK_RECONSTRUCT ? 2 * q.r.ticks : 2;
    }
    while (!pending_.empty()) {
        Request& q = reqs_[pending_.front()];
        const int qi = q.r.task == JC_TASK_RECONSTRUCT ? 2 * q.r.ticks : 2;
        if (cells + q.inst_cells() > max_cells_ || inst + qi > max_inst_ || used_bytes_ + q.bytes > budget_bytes_)
            break;  // first in, first admitted: later requests wait behind it
        pending_.pop_front();
        cells += q.inst_cells();
        inst += qi;
        used_bytes_ += q.bytes;
        q.admitted = true;
        q.fresh = true;
        q.t_admit = now_s();
        active_.push_back(q.id);
    }
}

void Server::loop() {
    std::vector<Request*> act;
    while (true) {
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
        }
        const double t0 = now_s();
        try {
            iteration(act);
        } catch (const std::exception& e) {
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
            cv_done_.notify_all();
            continue;
        }
        std::lock_guard<std::mutex> lk(mu_);
        busy_s_ += now_s() - t0;
        iterations_++;
        std::vector<uint64_t> still;
        for (Request* q : act) {
            if (q->finished) {
                q->done = true;
                completed_++;
                cell_ticks_ += (double)q->cells * q->r.ticks;
                last_done_ = q->t_done;
                used_bytes_ -= q->bytes;
            } else {
                still.push_back(q->id);
            }
        }
        active_.swap(still);
        cv_done_.notify_all();
    }
}

void Server::iteration(std::vector<Request*>& act) {
    cudaStream_t s = stream_;
    // new requests: buffers and inputs on the device
    for (Request* q : act)
        if (q->fresh && !q->d_state) allocate(*q);
    // descriptor lists: [init (new forward/rewind)] [forward group] [reverse group]
    std::vector<InstDev> init, fg, rg;
    std::vector<const Model*> fmod, rmod;
    auto base_inst = [&](const Model& m) {
        InstDev d{};
        d.tx = m.cfg.nx / m.cfg.patch;
        d.ty = m.cfg.ny / m.cfg.patch;
        d.nx = m.cfg.nx;
        d.ny = m.cfg.ny;
        d.pos = m.w.pos;
        return d;
    };
    for (Request* q : act) {
        const int g = q->r.grid;
        if (q->r.task == JC_TASK_RECONSTRUCT) {
            const size_t len = 3 * q->cells;
            for (int t = 1; t <= q->r.ticks; t++) {  // F_t = step_F(X_{t-1})
                InstDev d = base_inst(*fwd_[g]);
                d.state = q->d_state + (size_t)(t - 1) * len;
                d.out = q->d_F + (size_t)(t - 1) * len;
                d.meta = q->d_meta;
                d.flags = 4u;
                fg.push_back(d);
            }
            for (int t = 0; t < q->r.ticks; t++) {  // R_t = step_R(X_{t+1})
                InstDev d = base_inst(*rev_[g]);
                d.state = q->d_state + (size_t)(t + 1) * len;
                d.out = q->d_R + (size_t)t * len;
                d.meta = q->d_meta;
                d.flags = 4u;
                rg.push_back(d);
            }
        } else {
            const Model& m = q->r.task == JC_TASK_FORWARD ? *fwd_[g] : *rev_[g];
            InstDev d = base_inst(m);
            d.state = q->d_state;
            d.out = q->d_state;
            d.meta = q->d_meta;
            d.flags = q->r.flags;
            d.slot = q->d_slot;
            if (q->fresh) init.push_back(d);
            (q->r.task == JC_TASK_FORWARD ? fg : rg).push_back(d);
        }
    }
    // pack offsets per group
    auto layout = [&](std::vector<InstDev>& v, int& rows, long long& cells, int& tiles, int& tt, int& ct,
                      long long& maxc) {
        rows = 0;
        cells = 0;
        tiles = tt = ct = 0;
        maxc = 0;
        for (InstDev& d : v) {
            d.row0 = rows;
            d.cell0 = cells;
            d.tile0 = tiles;
            d.tt0 = tt;
            d.ct0 = ct;
            rows += d.tx * d.ty;
            cells += (long long)d.nx * d.ny;
            tiles += cell_tiles(d.nx, d.ny);
            tt += conv_tiles(d.tx, d.ty);
            ct += conv_tiles(d.nx, d.ny);
            maxc = std::max(maxc, (long long)d.nx * d.ny);
        }
    };
    int fr, ft, ftt, fct, rr, rt, rtt, rct, ir, it_, itt, ict;
    long long fc, rc, fmax, rmax, ic, imax;
    layout(fg, fr, fc, ft, ftt, fct, fmax);
    layout(rg, rr, rc, rt, rtt, rct, rmax);
    layout(init, ir, ic, it_, itt, ict, imax);
    const int n_all = (int)(init.size() + fg.size() + rg.size());
    if (n_all > max_inst_) throw Error(JC_OVER_BUDGET, "too many instances for the server's descriptor array");
    std::memcpy(h_inst_, init.data(), init.size() * sizeof(InstDev));
    std::memcpy(h_inst_ + init.size(), fg.data(), fg.size() * sizeof(InstDev));
    std::memcpy(h_inst_ + init.size() + fg.size(), rg.data(), rg.size() * sizeof(InstDev));
    cuda_check(cudaMemcpyAsync(ws_.base.inst, h_inst_, (size_t)n_all * sizeof(InstDev), cudaMemcpyHostToDevice, s),
               "descriptors", JC_MAP);
    const int fi = (int)init.size(), ri = fi + (int)fg.size();
    Pack pf = ws_.view(dims_, fi, (int)fg.size(), 0, fr, 0, fc, ft, ftt, fct);
    pf.max_inst_cells = fmax;
    Pack pr = ws_.view(dims_, ri, (int)rg.size(), fr, rr, fc, rc, rt, rtt, rct);
    pr.max_inst_cells = rmax;
    const BF16Path* bf = fwd_[0]->w.bf16.get();
    if (bf) {
        if (!fg.empty()) {
            bf->prepare(dims_, pf, h_inst_ + fi, s);
            bf->tune(dims_, fwd_[0]->w.f32, pf, s);
        }
        if (!rg.empty()) {
            bf->prepare(dims_, pr, h_inst_ + ri, s);
            rev_[0]->w.bf16->tune(dims_, rev_[0]->w.f32, pr, s);
        }
    }
    if (!init.empty()) {
        Pack pi = ws_.view(dims_, 0, (int)init.size(), 0, ir, 0, ic, it_, itt, ict);
        pi.max_inst_cells = imax;
        projection(dims_, pi, 1, s);
    }
    if (!fg.empty()) {
        fwd_[0]->forward_pack(pf, kWriteNextState, s);
        projection(dims_, pf, 0, s);
    }
    if (!rg.empty()) {
        rev_[0]->forward_pack(pr, kWriteNextState, s);
        projection(dims_, pr, 0, s);
    }
    std::vector<Request*> recon;
    for (Request* q : act) {
        q->fresh = false;
        if (q->r.task == JC_TASK_RECONSTRUCT) {
            cuda_check(cudaMemsetAsync(q->d_resid, 0, 4, s), "memset");
            recon_update_kernel<<<1024, 256, 0, s>>>(q->d_state, q->d_F, q->d_R, q->d_vals, q->d_known, q->r.ticks,
                                                     (long long)q->cells, q->d_resid);
            cuda_check(cudaGetLastError(), "recon update");
            recon.push_back(q);
        }
    }
    // results of forward/rewind requests that finish with this tick
    std::vector<Request*> finishing;
    for (Request* q : act) {
        if (q->r.task == JC_TASK_RECONSTRUCT) continue;
        if (q->ticks_done + 1 == q->r.ticks) {
            q->out.resize(3 * q->cells);
            cuda_check(cudaMemcpyAsync(q->out.data(), q->d_state, q->out.size() * 4, cudaMemcpyDeviceToHost, s), "D2H",
                       JC_MAP);
            finishing.push_back(q);
        }
    }
    std::vector<unsigned> resid(recon.size());
    std::vector<ProjSlot> slots(finishing.size());
    for (size_t i = 0; i < recon.size(); i++)
        cuda_check(cudaMemcpyAsync(&resid[i], recon[i]->d_resid, 4, cudaMemcpyDeviceToHost, s), "D2H", JC_MAP);
    for (size_t i = 0; i < finishing.size(); i++)
        cuda_check(cudaMemcpyAsync(&slots[i], finishing[i]->d_slot, sizeof(ProjSlot), cudaMemcpyDeviceToHost, s),
                   "D2H", JC_MAP);
    cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    ws_.check_timeout(s);
    const double t = now_s();
    for (size_t i = 0; i < finishing.size(); i++) {
        Request* q = finishing[i];
        q->energy = slots[i].energy;
        q->max_viol = slots[i].max_viol;
    }
    for (Request* q : act) {
        if (q->r.task != JC_TASK_RECONSTRUCT) {
            q->ticks_done++;
            if (q->ticks_done == q->r.ticks) {
                release(*q);
                q->finished = true;
                q->t_done = t;
            }
        }
    }
    for (size_t i = 0; i < recon.size(); i++) {
        Request* q = recon[i];
        q->sweeps++;
        float r;
        std::memcpy(&r, &resid[i], 4);
        q->residual = r;
        if (r < q->r.tol || q->sweeps >= q->r.max_sweeps) {
            q->out.resize((size_t)(q->r.ticks + 1) * 3 * q->cells);
            cuda_check(cudaMemcpyAsync(q->out.data(), q->d_state, q->out.size() * 4, cudaMemcpyDeviceToHost, s), "D2H",
                       JC_MAP);
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
            release(*q);
            q->finished = true;
            q->t_done = now_s();
        }
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
}  // namespace jc
