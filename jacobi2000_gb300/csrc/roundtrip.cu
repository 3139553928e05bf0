// Rewind round trip on the device: every trajectory runs N ticks with a
// forward checkpoint and then N ticks with its reverse checkpoint, and the
// result is scored against the start: correlation over (h, u, v) and
// amplitude ratio (metrics.rs:9-27), the round-trip RMSE (metrics.rs:109-112)
// and the RMSE of the N-tick change itself, the score a do-nothing rewind
// would get (the round-trip runs of docs/runs/2026-09-20-rewind-round-trip.md:
// 17-32). The forward rollouts of all trajectories are one batch; a tick hook
// copies their states at each horizon; the reverse rollouts of all
// (horizon, trajectory) pairs, with their uneven lengths, are a second batch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "evaluate.hpp"

namespace jc {
namespace rt {

constexpr int kThreads = 512;

// Copies state k (src[k], len floats, len % 4 == 0) to dst + k * len.
__global__ void __launch_bounds__(kThreads) snap_kernel(const float* const* src, float* dst, long long len) {
    const int k = blockIdx.y;
    const float4* s = reinterpret_cast<const float4*>(src[k]);
    float4* d = reinterpret_cast<float4*>(dst + (long long)k * len);
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < len / 4; i += (long long)gridDim.x * kThreads)
        d[i] = s[i];
}

struct RtRec {
    double sab, saa, sbb;  // correlation sums of (rewound state, start state)
    double se_rt, se_chg;  // squared errors: rewound - start, N-tick state - start
    float peak_y, peak_x;  // max |h| (decoded) of the rewound and the start state
};

template <int N>
__device__ void block_sum(double (&v)[N], double* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = warp_sum_d(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++) red[k * 32 + w] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = warp_sum_d(lane < nw ? red[k * 32 + lane] : 0.0);
    __syncthreads();
}

__device__ float block_max(float v, float* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    float t = lane < nw ? red[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    __syncthreads();
    return t;
}

// One CTA per (horizon, trajectory) slot s: y = rewound state, xn = state
// after the forward ticks, x0 = start state of trajectory s % n.
__global__ void __launch_bounds__(kThreads)
score_kernel(const float* y_all, const float* xn_all, long long slot_stride, const float* x0_all, int n,
             long long len, long long cells, float std0, float mean0, RtRec* recs) {
    __shared__ double red[5 * 32];
    __shared__ float fred[32];
    const int s = blockIdx.x;
    const float* y = y_all + (long long)s * slot_stride;
    const float* xn = xn_all + (long long)s * slot_stride;
    const float* x0 = x0_all + (long long)(s % n) * len;
    double s1[2] = {0.0, 0.0};
    float py = 0.f, px = 0.f;
    for (long long i = threadIdx.x; i < len; i += kThreads) {
        const float a = y[i], b = x0[i];
        s1[0] += (double)a;
        s1[1] += (double)b;
        if (i < cells) {
            py = fmaxf(py, fabsf(__fadd_rn(__fmul_rn(a, std0), mean0)));
            px = fmaxf(px, fabsf(__fadd_rn(__fmul_rn(b, std0), mean0)));
        }
    }
    block_sum(s1, red);
    py = block_max(py, fred);
    px = block_max(px, fred);
    const double ma = s1[0] / (double)len, mb = s1[1] / (double)len;
    double s2[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (long long i = threadIdx.x; i < len; i += kThreads) {
        const float a = y[i], b = x0[i], c = xn[i];
        const double da = __dsub_rn((double)a, ma), db = __dsub_rn((double)b, mb);
        s2[0] = __dadd_rn(s2[0], __dmul_rn(da, db));
        s2[1] = __dadd_rn(s2[1], __dmul_rn(da, da));
        s2[2] = __dadd_rn(s2[2], __dmul_rn(db, db));
        const double e1 = (double)__fsub_rn(a, b), e2 = (double)__fsub_rn(c, b);
        s2[3] = __dadd_rn(s2[3], __dmul_rn(e1, e1));
        s2[4] = __dadd_rn(s2[4], __dmul_rn(e2, e2));
    }
    block_sum(s2, red);
    if (threadIdx.x == 0) {
        RtRec r;
        r.sab = s2[0];
        r.saa = s2[1];
        r.sbb = s2[2];
        r.se_rt = s2[3];
        r.se_chg = s2[4];
        r.peak_y = py;
        r.peak_x = px;
        recs[s] = r;
    }
}

class RoundTrip : public TickHook {
   public:
    RoundTrip(jc_model* fwd, jc_model* rev, int max_traj, int max_h) : max_(max_traj), max_h_(max_h) {
        if (max_traj < 1 || max_h < 1) throw Error(JC_BAD_ARGUMENT, "max_trajectories and max_horizons must be >= 1");
        const jc_config &a = fwd->m->cfg, &b = rev->m->cfg;
        if (a.nx != b.nx || a.ny != b.ny) throw Error(JC_BAD_SHAPE, "forward and reverse checkpoints differ in grid");
        cfg_ = a;
        cells_ = (long long)a.nx * a.ny;
        len_ = 3 * cells_;
        jc_model* list[2] = {fwd, rev};
        const long long slots = (long long)max_traj * max_h;
        if (slots > (1 << 30)) throw Error(JC_BAD_ARGUMENT, "too many trajectories x horizons");
        batch_.reset(new Batch(list, 2, (int)slots, slots * cells_));
        cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        x0_ = arena_.alloc_n<float>(max_ * len_);
        fin_ = arena_.alloc_n<float>(max_ * len_);
        snap_ = arena_.alloc_n<float>(slots * len_);
        back_ = arena_.alloc_n<float>(slots * len_);
        src_ = arena_.alloc_n<const float*>(max_);
        recs_ = arena_.alloc_n<RtRec>(slots);
        meta_ = arena_.alloc_n<float>(128);
        std::vector<float> meta(128, 0.f);
        fwd->m->meta_of(meta.data());
        rev->m->meta_of(meta.data() + 64);
        cuda_check(cudaMemcpy(meta_, meta.data(), 128 * 4, cudaMemcpyHostToDevice), "meta upload", JC_MAP);
        cuda_check(cudaMallocHost(&h_phys_, 2 * max_ * len_ * sizeof(float)), "cudaMallocHost", JC_OVER_BUDGET);
    }
    ~RoundTrip() override {
        if (h_phys_) cudaFreeHost(h_phys_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    void run(const jc_drop* drops, int n, const int32_t* horizons, int nh, uint32_t flags, jc_roundtrip_row* rows) {
        if (n < 1 || n > max_) throw Error(JC_BAD_ARGUMENT, "trajectory count outside [1, max_trajectories]");
        if (nh < 1 || nh > max_h_) throw Error(JC_BAD_ARGUMENT, "horizon count outside [1, max_horizons]");
        if (!drops || !horizons || !rows) throw Error(JC_BAD_ARGUMENT, "null argument");
        if (flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown flag");
        for (int i = 0; i < nh; i++)
            if (horizons[i] < 1 || (i > 0 && horizons[i] <= horizons[i - 1]))
                throw Error(JC_BAD_ARGUMENT, "horizons must be >= 1 and strictly ascending");
        n_ = n;
        horizons_.assign(horizons, horizons + nh);
        float* P = h_phys_;
        float* X = h_phys_ + max_ * len_;
        for (int k = 0; k < n; k++) ev::initial_state(cfg_, drops[k], P + k * len_, X + k * len_);
        cuda_check(cudaMemcpyAsync(x0_, X, n * len_ * sizeof(float), cudaMemcpyHostToDevice, stream_), "H2D", JC_MAP);
        // forward: every trajectory to the last horizon, states copied at each horizon
        std::vector<jc_instance> fw(n);
        std::vector<double> energy(2 * (size_t)n * (nh + 1), 0.0);
        for (int k = 0; k < n; k++) {
            jc_instance& I = fw[k];
            std::memset(&I, 0, sizeof(I));
            I.model = 0;
            I.ticks = horizons_.back();
            I.flags = flags;
            I.x0 = x0_ + k * len_;
            I.meta = meta_;
            I.final_state = fin_ + k * len_;
            I.energy = &energy[2 * k];
        }
        batch_->rollout(fw.data(), n, true, stream_, this);
        // reverse: each (horizon, trajectory) state back by its horizon
        std::vector<jc_instance> rv((size_t)nh * n);
        for (int i = 0; i < nh; i++)
            for (int k = 0; k < n; k++) {
                const size_t slot = (size_t)i * n + k;
                jc_instance& I = rv[slot];
                std::memset(&I, 0, sizeof(I));
                I.model = 1;
                I.ticks = horizons_[i];
                I.flags = flags;
                I.x0 = snap_ + slot * len_;
                I.meta = meta_ + 64;
                I.final_state = back_ + slot * len_;
                I.energy = &energy[2 * (n + slot)];
            }
        batch_->rollout(rv.data(), nh * n, true, stream_, nullptr);
        {
            KScope ks("roundtrip_score", stream_);
            score_kernel<<<nh * n, kThreads, 0, stream_>>>(back_, snap_, len_, x0_, n, len_, cells_,
                                                           cfg_.norm_std[0], cfg_.norm_mean[0], recs_);
            cuda_check(cudaGetLastError(), "roundtrip score launch");
        }
        std::vector<RtRec> rec((size_t)nh * n);
        cuda_check(cudaMemcpyAsync(rec.data(), recs_, rec.size() * sizeof(RtRec), cudaMemcpyDeviceToHost, stream_),
                   "D2H", JC_MAP);
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize", JC_POLL);
        for (size_t s = 0; s < rec.size(); s++) {
            const RtRec& r = rec[s];
            jc_roundtrip_row& o = rows[s];
            o.corr = (r.saa <= 0.0 || r.sbb <= 0.0) ? 0.0f : (float)(r.sab / std::sqrt(r.saa * r.sbb));
            o.amplitude_ratio = r.peak_y / r.peak_x;
            o.rmse = (float)std::sqrt(r.se_rt / (double)len_);
            o.change_rmse = (float)std::sqrt(r.se_chg / (double)len_);
        }
    }

    void bind(const std::vector<float*>& states, cudaStream_t s) override {
        cuda_check(cudaMemcpyAsync(src_, states.data(), states.size() * sizeof(float*), cudaMemcpyHostToDevice, s),
                   "state pointers", JC_MAP);
        cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    }

    void after_tick(int t, cudaStream_t s) const override {
        for (size_t i = 0; i < horizons_.size(); i++)
            if (horizons_[i] == t) {
                KScope ks("roundtrip_snap", s);
                const long long blocks = std::min<long long>((len_ / 4 + kThreads - 1) / kThreads, 64);
                // slot (i, k) lives at snap_ + (i n + k) len
                snap_kernel<<<dim3((unsigned)blocks, n_), kThreads, 0, s>>>(src_, snap_ + (long long)i * n_ * len_,
                                                                          len_);
                cuda_check(cudaGetLastError(), "roundtrip snapshot launch");
            }
    }

    long long key() const override {
        unsigned long long h = 1469598103934665603ull;
        auto mix = [&](unsigned long long v) { h = (h ^ v) * 1099511628211ull; };
        mix((unsigned long long)(uintptr_t)this);
        mix((unsigned long long)n_);
        for (int hz : horizons_) mix((unsigned long long)hz);
        return (long long)(h >> 1);
    }

   private:
    int max_, max_h_;
    jc_config cfg_{};
    long long cells_ = 0, len_ = 0;
    std::unique_ptr<Batch> batch_;
    cudaStream_t stream_ = nullptr;
    DeviceArena arena_;
    float *x0_ = nullptr, *fin_ = nullptr, *snap_ = nullptr, *back_ = nullptr, *meta_ = nullptr;
    const float** src_ = nullptr;
    RtRec* recs_ = nullptr;
    float* h_phys_ = nullptr;
    int n_ = 0;
    std::vector<int> horizons_;
};

}  // namespace rt
}  // namespace jc

struct jc_roundtrip {
    jc::rt::RoundTrip* r;
};

namespace jc {
jc_roundtrip* roundtrip_create(jc_model* fwd, jc_model* rev, int max_traj, int max_h) {
    return new jc_roundtrip{new rt::RoundTrip(fwd, rev, max_traj, max_h)};
}
void roundtrip_destroy(jc_roundtrip* r) {
    delete r->r;
    delete r;
}
void roundtrip_run(jc_roundtrip* r, const jc_drop* drops, int n, const int32_t* horizons, int nh, uint32_t flags,
                   jc_roundtrip_row* rows) {
    r->r->run(drops, n, horizons, nh, flags, rows);
}
}  // namespace jc
