// The extern "C" surface (include/jacobi2000.h). Every entry point catches
// all exceptions and returns a status; the message is kept per thread.
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/jacobi2000.h"
#include "bf16_path.hpp"
#include "runtime.hpp"

namespace {
thread_local std::string g_last_error;

jc_status fail(jc_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

template <class F>
jc_status guard(F&& f) {
    try {
        f();
        g_last_error.clear();
        return JC_OK;
    } catch (const jc::Error& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(JC_OVER_BUDGET, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(JC_CUDA_ERROR, e.what());
    } catch (...) {
        return fail(JC_CUDA_ERROR, "unknown error");
    }
}

struct Neu {
    double s = 0.0, c = 0.0;
    void add(double v) {
        double t = s + v;
        if (std::fabs(s) >= std::fabs(v)) c += (s - t) + v; else c += (v - t) + s;
        s = t;
    }
    double val() const { return s + c; }
};

// project.rs:9-19: per-cell terms in f32 as the reference forms them (this
// file is compiled without multiply-add contraction), accumulated in f64 with
// Neumaier compensation.
void pk(const float* x, const jc_config* c, int64_t n, double* P, double* K) {
    Neu p, k;
    const float hoff = c->norm_mean[0] + c->norm_depth;
    for (int64_t i = 0; i < n; i++) {
        float h = x[i] * c->norm_std[0] + hoff;
        float u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        float v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        p.add((double)(0.5f * c->g * h * h));
        k.add((double)(0.5f * h * (u * u + v * v)));
    }
    *P = p.val();
    *K = k.val();
}
}  // namespace

extern "C" {

jc_status jc_model_create(const uint8_t* st, size_t st_len, const char* config_json, int32_t precision,
                          jc_model** out) {
    if (!out) return fail(JC_BAD_ARGUMENT, "out is null");
    *out = nullptr;
    return guard([&] {
        jc::Model* m = new jc::Model(st, st_len, config_json, precision);
        *out = new jc_model{m};
    });
}

jc_status jc_model_pack(const jc_model* m, uint8_t* buf, size_t cap, size_t* len) {
    if (!m || !len) return fail(JC_BAD_ARGUMENT, "null argument");
    return guard([&] {
        std::vector<uint8_t> p = m->m->pack();
        *len = p.size();
        if (buf) {
            if (cap < p.size()) throw jc::Error(JC_LIMIT, "buffer smaller than the pre-packed checkpoint");
            std::memcpy(buf, p.data(), p.size());
        }
    });
}

jc_status jc_model_create_packed(const uint8_t* packed, size_t len, jc_model** out) {
    if (!out) return fail(JC_BAD_ARGUMENT, "out is null");
    *out = nullptr;
    return guard([&] {
        jc::Model* m = new jc::Model(packed, len);
        *out = new jc_model{m};
    });
}

jc_status jc_source_hash(const uint8_t* st, size_t st_len, const char* config_json, uint64_t* out) {
    if (!st || !config_json || !out) return fail(JC_BAD_ARGUMENT, "null argument");
    return guard([&] { *out = jc::source_hash(st, st_len, config_json); });
}

jc_status jc_packed_source_hash(const uint8_t* packed, size_t len, uint64_t* out) {
    if (!out) return fail(JC_BAD_ARGUMENT, "null argument");
    return guard([&] { *out = jc::packed_source_hash(packed, len); });
}

void jc_model_destroy(jc_model* m) {
    if (!m) return;
    try {
        delete m->m;
    } catch (...) {
    }
    delete m;
}

jc_status jc_model_config(const jc_model* m, jc_config* out) {
    if (!m || !out) return fail(JC_BAD_ARGUMENT, "null argument");
    *out = m->m->cfg;
    return JC_OK;
}

jc_status jc_meta_of(const jc_model* m, float* meta_out) {
    if (!m || !meta_out) return fail(JC_BAD_ARGUMENT, "null argument");
    m->m->meta_of(meta_out);
    return JC_OK;
}

jc_status jc_forward(jc_model* m, const float* state, const float* meta, float* increment) {
    if (!m) return fail(JC_BAD_ARGUMENT, "model is null");
    return guard([&] { m->m->forward_host(state, meta, increment); });
}

jc_status jc_step(jc_model* m, const float* state, const float* meta, float* next_state) {
    if (!m) return fail(JC_BAD_ARGUMENT, "model is null");
    return guard([&] { m->m->step_host(state, meta, next_state); });
}

jc_status jc_rollout(jc_model* m, const float* x0, const float* meta, int32_t ticks, uint32_t flags,
                     float* final_state, float* trajectory, double* energies) {
    if (!m) return fail(JC_BAD_ARGUMENT, "model is null");
    return guard([&] { m->m->rollout_host(x0, meta, ticks, flags, final_state, trajectory, energies); });
}

jc_status jc_forward_device(jc_model* m, const float* d_state, const float* d_meta, float* d_increment,
                            void* stream) {
    if (!m) return fail(JC_BAD_ARGUMENT, "model is null");
    return guard([&] { m->m->forward_device(d_state, d_meta, d_increment, (cudaStream_t)stream); });
}

jc_status jc_rollout_device(jc_model* m, const float* d_x0, const float* d_meta, int32_t ticks, uint32_t flags,
                            float* d_final, double* d_energies, void* stream) {
    if (!m) return fail(JC_BAD_ARGUMENT, "model is null");
    if (!d_x0 || !d_meta) return fail(JC_BAD_ARGUMENT, "null buffer");
    return guard([&] { m->m->rollout_device(d_x0, d_meta, ticks, flags, d_final, d_energies, (cudaStream_t)stream); });
}

jc_status jc_forward_device_noalloc(jc_model* m, const float* d_state, const float* d_meta, float* d_increment,
                                    void* stream) {
    if (!m) return fail(JC_BAD_ARGUMENT, "model is null");
    return guard([&] { jc::forward_noalloc(*m->m, d_state, d_meta, d_increment, (cudaStream_t)stream); });
}

jc_status jc_selftest_device_wait(int32_t satisfy, uint32_t limit_us) {
    return guard([&] { jc::selftest_device_wait(satisfy, limit_us); });
}

jc_status jc_batch_create(jc_model* const* models, int32_t n_models, int32_t max_instances, int64_t max_cells,
                          jc_batch** out) {
    if (!out) return fail(JC_BAD_ARGUMENT, "out is null");
    *out = nullptr;
    return guard([&] {
        jc::Batch* b = new jc::Batch(models, n_models, max_instances, max_cells);
        *out = new jc_batch{b};
    });
}

void jc_batch_destroy(jc_batch* b) {
    if (!b) return;
    try {
        delete b->b;
    } catch (...) {
    }
    delete b;
}

jc_status jc_batch_rollout(jc_batch* b, const jc_instance* instances, int32_t n, int32_t device_pointers,
                           void* stream) {
    if (!b) return fail(JC_BAD_ARGUMENT, "batch is null");
    return guard([&] { b->b->rollout(instances, n, device_pointers != 0, (cudaStream_t)stream); });
}

jc_status jc_server_create(jc_model* const* forward_models, jc_model* const* reverse_models, int32_t n_grids,
                           int64_t max_active_cells, double hbm_fraction, jc_server** out) {
    if (!out) return fail(JC_BAD_ARGUMENT, "out is null");
    *out = nullptr;
    return guard([&] { jc::server_create(forward_models, reverse_models, n_grids, max_active_cells, hbm_fraction, out); });
}

void jc_server_destroy(jc_server* s) {
    if (!s) return;
    try {
        jc::server_destroy(s);
    } catch (...) {
    }
}

jc_status jc_server_submit(jc_server* s, const jc_request* r, uint64_t* id) {
    if (!s || !r || !id) return fail(JC_BAD_ARGUMENT, "null argument");
    return guard([&] { *id = jc::server_submit(s, r); });
}

jc_status jc_server_wait(jc_server* s, uint64_t id, float* out, size_t out_len, jc_result* info, double timeout_s) {
    if (!s) return fail(JC_BAD_ARGUMENT, "server is null");
    return guard([&] { jc::server_wait(s, id, out, out_len, info, timeout_s); });
}

jc_status jc_server_get_stats(jc_server* s, jc_server_stats* out) {
    if (!s || !out) return fail(JC_BAD_ARGUMENT, "null argument");
    return guard([&] { jc::server_stats(s, out); });
}

jc_status jc_server_reset_stats(jc_server* s) {
    if (!s) return fail(JC_BAD_ARGUMENT, "server is null");
    return guard([&] { jc::server_reset_stats(s); });
}

jc_status jc_server_profile(jc_server* s, int32_t enable, char* report, size_t cap) {
    if (!s) return fail(JC_BAD_ARGUMENT, "server is null");
    return guard([&] { jc::server_profile(s, enable, report, cap); });
}

jc_status jc_batch_profile(jc_batch* b, const jc_instance* instances, int32_t n, int32_t device_pointers,
                           char* report, size_t cap) {
    if (!b || !report || cap == 0) return fail(JC_BAD_ARGUMENT, "null argument");
    return guard([&] {
        auto s = b->b->profile(instances, n, device_pointers != 0);
        std::string out;
        for (auto& kv : s)
            out += kv.first + "," + std::to_string(kv.second.first) + "," + std::to_string(kv.second.second) + "\n";
        size_t k = std::min(out.size(), cap - 1);
        std::memcpy(report, out.data(), k);
        report[k] = '\0';
    });
}

double jc_mass(const float* x, int64_t n) {
    if (!x || n <= 0) return 0.0;
    Neu s;
    for (int64_t i = 0; i < n; i++) s.add((double)x[i]);
    return s.val() / (double)n;
}

double jc_energy(const float* x, const jc_config* cfg, int64_t n) {
    if (!x || !cfg || n <= 0) return 0.0;
    double P, K;
    pk(x, cfg, n, &P, &K);
    return P + K;
}

void jc_project_mass(float* x, double target, int64_t n) {
    if (!x || n <= 0) return;
    float delta = (float)(target - jc_mass(x, n));
    for (int64_t i = 0; i < n; i++) x[i] += delta;
}

void jc_project_energy(float* x, double prev_energy, const jc_config* c, int64_t n) {
    if (!x || !c || n <= 0) return;
    double P, K;
    pk(x, c, n, &P, &K);
    double budget = prev_energy * (double)c->energy_r_max - P;
    if (!(budget > 0.0)) budget = 0.0;
    double s = std::sqrt(budget / (K > 1e-12 ? K : 1e-12));
    float s32 = (float)(s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s));
    for (int64_t i = 0; i < n; i++) {
        float u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        float v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        x[n + i] = (u * s32 - c->norm_mean[1]) / c->norm_std[1];
        x[2 * n + i] = (v * s32 - c->norm_mean[2]) / c->norm_std[2];
    }
}

jc_status jc_sw_run(const jc_sw_params* p, float* states, int32_t count, int32_t steps) {
    if (!p) return fail(JC_BAD_ARGUMENT, "params are null");
    return guard([&] { jc::sw_run_host(*p, states, count, steps); });
}

jc_status jc_sw_run_device(const jc_sw_params* p, float* d_states, int32_t count, int32_t steps, void* stream) {
    if (!p) return fail(JC_BAD_ARGUMENT, "params are null");
    return guard([&] { jc::sw_run_device(*p, d_states, count, steps, (cudaStream_t)stream); });
}

jc_status jc_sw_trajectories(const jc_sw_params* p, const jc_sw_trajectory* t, int32_t n) {
    if (!p) return fail(JC_BAD_ARGUMENT, "params are null");
    return guard([&] { jc::sw_trajectories_host(*p, t, n); });
}

jc_status jc_sw_add_drop(const jc_sw_params* p, float* h, float cx, float cy, float amp, float sigma) {
    if (!p) return fail(JC_BAD_ARGUMENT, "params are null");
    return guard([&] { jc::sw_add_drop_host(*p, h, cx, cy, amp, sigma); });
}

jc_status jc_eval_score(const jc_config* cfg, const float* x, const float* truth, const float* centres,
                        int32_t count, jc_eval_row* rows) {
    if (!cfg) return fail(JC_BAD_ARGUMENT, "config is null");
    return guard([&] { jc::eval_score_host(*cfg, x, truth, centres, count, rows); });
}

jc_status jc_eval_create(jc_model* m, int32_t max_trajectories, jc_eval** out) {
    if (!m || !out) return fail(JC_BAD_ARGUMENT, "null argument");
    *out = nullptr;
    return guard([&] { *out = jc::eval_create(m, max_trajectories); });
}

void jc_eval_destroy(jc_eval* e) {
    if (!e) return;
    try {
        jc::eval_destroy(e);
    } catch (...) {
    }
}

jc_status jc_eval_run(jc_eval* e, const jc_drop* drops, int32_t n, const int32_t* horizons, int32_t n_horizons,
                      uint32_t flags, jc_eval_row* rows, double* max_violation) {
    if (!e) return fail(JC_BAD_ARGUMENT, "evaluator is null");
    return guard([&] { jc::eval_run(e, drops, n, horizons, n_horizons, flags, rows, max_violation); });
}

jc_status jc_roundtrip_create(jc_model* forward, jc_model* reverse, int32_t max_trajectories, int32_t max_horizons,
                              jc_roundtrip** out) {
    if (!forward || !reverse || !out) return fail(JC_BAD_ARGUMENT, "null argument");
    *out = nullptr;
    return guard([&] { *out = jc::roundtrip_create(forward, reverse, max_trajectories, max_horizons); });
}

void jc_roundtrip_destroy(jc_roundtrip* r) {
    if (!r) return;
    try {
        jc::roundtrip_destroy(r);
    } catch (...) {
    }
}

jc_status jc_roundtrip_run(jc_roundtrip* r, const jc_drop* drops, int32_t n, const int32_t* horizons,
                           int32_t n_horizons, uint32_t flags, jc_roundtrip_row* rows) {
    if (!r) return fail(JC_BAD_ARGUMENT, "round trip is null");
    return guard([&] { jc::roundtrip_run(r, drops, n, horizons, n_horizons, flags, rows); });
}

const char* jc_last_error(void) { return g_last_error.c_str(); }

int32_t jc_autotune(int32_t enable) {
    const int prev = jc::g_autotune.load();
    if (enable >= 0) jc::g_autotune.store(enable ? 1 : 0);
    return prev;
}

const char* jc_version(void) { return "jacobi2000-gb300 0.1 (sm_103a)"; }

}  // extern "C"
