/*
 * CPU oracle: instantiates the forward pass for f32 and f64 and restates the
 * reference's projections and tick loop. TEST INFRASTRUCTURE ONLY: see
 * oracle.h. Build with -ffp-contract=off so no multiply-add is fused (the
 * reference's Rust arithmetic is unfused), which keeps results identical on
 * x86-64 and aarch64.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_attention_mode = 1;

void orc_set_attention_mode(int mode) { g_attention_mode = mode; }

void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* mask.rs:18-30 — Chebyshev box with dilation; truncated division as Rust's
 * isize `/` and `%`. */
static int mask_allowed(const orc_config* c, int tx, int q, int k) {
    if (c->mask_kind == 0) return 1;
    int qx = q % tx, qy = q / tx, kx = k % tx, ky = k / tx;
    int dx = kx - qx, dy = ky - qy, d = c->dilation;
    if (dx % d != 0 || dy % d != 0) return 0;
    int ax = dx / d, ay = dy / d;
    if (ax < 0) ax = -ax;
    if (ay < 0) ay = -ay;
    return ax <= c->radius && ay <= c->radius;
}

/* ---- f32: the reference's arithmetic ---- */
#define R float
#define FN(name) name##_f32
#define SQRTR sqrtf
#define EXPR expf
#define ERFR erff
/* std::f32::consts::SQRT_2.recip(), rounded in f32 (cpu.rs:70) */
#define INV_SQRT2 (1.0f / 1.41421356237309504880f)
#define LN_EPS 1e-5f
#include "oracle_impl.inc"
#undef R
#undef FN
#undef SQRTR
#undef EXPR
#undef ERFR
#undef INV_SQRT2
#undef LN_EPS

/* ---- f64: the same algorithm in double precision ---- */
#define R double
#define FN(name) name##_f64
#define SQRTR sqrt
#define EXPR exp
#define ERFR erf
#define INV_SQRT2 (0.70710678118654752440)
#define LN_EPS 1e-5
#include "oracle_impl.inc"
#undef R
#undef FN
#undef SQRTR
#undef EXPR
#undef ERFR
#undef INV_SQRT2
#undef LN_EPS

/* ---- projections, f32 sequential sums: project.rs:9-54 ---- */

static void pk_f32(const float* x, const orc_config* c, int n, float* p, float* k) {
    float pot = 0.0f, kin = 0.0f;
    const float h_off = c->norm_mean[0] + c->norm_depth;
    for (int i = 0; i < n; i++) {
        float h = x[i] * c->norm_std[0] + h_off;
        float u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        float v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        pot += 0.5f * c->g * h * h;
        kin += 0.5f * h * (u * u + v * v);
    }
    *p = pot;
    *k = kin;
}

float orc_energy_f32(const float* x, const orc_config* c, int n) {
    float p, k;
    pk_f32(x, c, n, &p, &k);
    return p + k;
}

float orc_mass_f32(const float* x, int n) {
    float s = 0.0f;
    for (int i = 0; i < n; i++) s += x[i];
    return s / (float)n;
}

void orc_project_mass_f32(float* x, float target, int n) {
    float delta = target - orc_mass_f32(x, n);
    for (int i = 0; i < n; i++) x[i] += delta;
}

static float clampf01(float s) { return s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s); }

void orc_project_energy_f32(float* x, float prev_energy, const orc_config* c, int n) {
    float bound = prev_energy * c->energy_r_max;
    float p, k;
    pk_f32(x, c, n, &p, &k);
    float budget = bound - p;
    if (!(budget > 0.0f)) budget = 0.0f;
    float kf = k > 1e-12f ? k : 1e-12f;
    float scale = clampf01(sqrtf(budget / kf));
    for (int i = 0; i < n; i++) {
        float u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        float v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        x[n + i] = (u * scale - c->norm_mean[1]) / c->norm_std[1];
        x[2 * n + i] = (v * scale - c->norm_mean[2]) / c->norm_std[2];
    }
}

/* ---- projections with f64 compensated (Neumaier) sums ----
 * The same formulas; every per-cell term is formed in f32 as the reference
 * forms it and summed in f64 with Neumaier compensation; the resulting shift
 * and scale are rounded to f32 and applied with the reference's f32 update. */

typedef struct { double s, c; } nsum;
static void nadd(nsum* a, double v) {
    double t = a->s + v;
    if (fabs(a->s) >= fabs(v)) a->c += (a->s - t) + v;
    else a->c += (v - t) + a->s;
    a->s = t;
}
static double nval(const nsum* a) { return a->s + a->c; }

static void pk_sum64(const float* x, const orc_config* c, int n, double* p, double* k) {
    /* per-cell terms exactly as project.rs:9-19 computes them (f32); only the
     * accumulation is f64 */
    nsum ps = {0, 0}, ks = {0, 0};
    const float h_off = c->norm_mean[0] + c->norm_depth;
    for (int i = 0; i < n; i++) {
        float h = x[i] * c->norm_std[0] + h_off;
        float u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        float v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        nadd(&ps, (double)(0.5f * c->g * h * h));
        nadd(&ks, (double)(0.5f * h * (u * u + v * v)));
    }
    *p = nval(&ps);
    *k = nval(&ks);
}

double orc_energy_sum64(const float* x, const orc_config* c, int n) {
    double p, k;
    pk_sum64(x, c, n, &p, &k);
    return p + k;
}

double orc_mass_sum64(const float* x, int n) {
    nsum s = {0, 0};
    for (int i = 0; i < n; i++) nadd(&s, (double)x[i]);
    return nval(&s) / (double)n;
}

void orc_project_mass_sum64(float* x, double target, int n) {
    float delta = (float)(target - orc_mass_sum64(x, n));
    for (int i = 0; i < n; i++) x[i] += delta;
}

void orc_project_energy_sum64(float* x, double prev_energy, const orc_config* c, int n) {
    double bound = prev_energy * (double)c->energy_r_max;
    double p, k;
    pk_sum64(x, c, n, &p, &k);
    double budget = bound - p;
    if (!(budget > 0.0)) budget = 0.0;
    double s = sqrt(budget / (k > 1e-12 ? k : 1e-12));
    float scale = (float)(s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s));
    for (int i = 0; i < n; i++) {
        float u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        float v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        x[n + i] = (u * scale - c->norm_mean[1]) / c->norm_std[1];
        x[2 * n + i] = (v * scale - c->norm_mean[2]) / c->norm_std[2];
    }
}

/* ---- projections in f64 for the f64 tick loop ---- */

static void pk_f64(const double* x, const orc_config* c, int n, double* p, double* k) {
    nsum ps = {0, 0}, ks = {0, 0};
    const double h_off = (double)c->norm_mean[0] + (double)c->norm_depth;
    for (int i = 0; i < n; i++) {
        double h = x[i] * c->norm_std[0] + h_off;
        double u = x[n + i] * c->norm_std[1] + c->norm_mean[1];
        double v = x[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
        nadd(&ps, 0.5 * (double)c->g * h * h);
        nadd(&ks, 0.5 * h * (u * u + v * v));
    }
    *p = nval(&ps);
    *k = nval(&ks);
}

static double mass_f64(const double* x, int n) {
    nsum s = {0, 0};
    for (int i = 0; i < n; i++) nadd(&s, x[i]);
    return nval(&s) / (double)n;
}

/* ---- tick loops: eval.rs:144-157 ---- */

double orc_rollout_f32(const orc_config* c, const orc_weights* w, const float* x0,
                       const float* meta, int ticks, unsigned flags, float* traj,
                       float* final_state, double* energies) {
    const int n = c->nx * c->ny;
    const size_t len = (size_t)c->channels * n;
    const int sum64 = (flags & ORC_SUM64) != 0;
    float* x = (float*)malloc(sizeof(float) * len);
    float* inc = (float*)malloc(sizeof(float) * len);
    memcpy(x, x0, sizeof(float) * len);
    if (traj) memcpy(traj, x, sizeof(float) * len);
    double mass0 = sum64 ? orc_mass_sum64(x, n) : (double)orc_mass_f32(x, n);
    double energy = sum64 ? orc_energy_sum64(x, c, n) : (double)orc_energy_f32(x, c, n);
    if (energies) energies[0] = energy;
    double max_violation = 0.0;
    for (int t = 1; t <= ticks; t++) {
        double prev = energy;
        orc_forward_f32(c, w, x, meta, inc);
        for (size_t i = 0; i < len; i++) inc[i] += x[i];          /* cpu.rs:84-88 */
        if (flags & ORC_MASS) {
            if (sum64) orc_project_mass_sum64(inc, mass0, n);
            else orc_project_mass_f32(inc, (float)mass0, n);
        }
        if (flags & ORC_ENERGY) {
            if (sum64) orc_project_energy_sum64(inc, prev, c, n);
            else orc_project_energy_f32(inc, (float)prev, c, n);
        }
        memcpy(x, inc, sizeof(float) * len);
        energy = sum64 ? orc_energy_sum64(x, c, n) : (double)orc_energy_f32(x, c, n);
        if (energies) energies[t] = energy;
        double viol = (energy - prev * (double)c->energy_r_max) / prev;
        if (viol > max_violation) max_violation = viol;
        if (traj) memcpy(traj + (size_t)t * len, x, sizeof(float) * len);
    }
    if (final_state) memcpy(final_state, x, sizeof(float) * len);
    free(x);
    free(inc);
    return max_violation;
}

double orc_rollout_f64(const orc_config* c, const orc_weights* w, const double* x0,
                       const double* meta, int ticks, unsigned flags, double* traj,
                       double* final_state, double* energies) {
    const int n = c->nx * c->ny;
    const size_t len = (size_t)c->channels * n;
    double* x = (double*)malloc(sizeof(double) * len);
    double* inc = (double*)malloc(sizeof(double) * len);
    memcpy(x, x0, sizeof(double) * len);
    if (traj) memcpy(traj, x, sizeof(double) * len);
    double mass0 = mass_f64(x, n);
    double p, k;
    pk_f64(x, c, n, &p, &k);
    double energy = p + k;
    if (energies) energies[0] = energy;
    double max_violation = 0.0;
    for (int t = 1; t <= ticks; t++) {
        double prev = energy;
        orc_forward_f64(c, w, x, meta, inc);
        for (size_t i = 0; i < len; i++) inc[i] += x[i];
        if (flags & ORC_MASS) {
            double delta = mass0 - mass_f64(inc, n);
            for (int i = 0; i < n; i++) inc[i] += delta;
        }
        if (flags & ORC_ENERGY) {
            double bound = prev * (double)c->energy_r_max;
            pk_f64(inc, c, n, &p, &k);
            double budget = bound - p;
            if (!(budget > 0.0)) budget = 0.0;
            double s = sqrt(budget / (k > 1e-12 ? k : 1e-12));
            s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
            for (int i = 0; i < n; i++) {
                double u = inc[n + i] * c->norm_std[1] + c->norm_mean[1];
                double v = inc[2 * n + i] * c->norm_std[2] + c->norm_mean[2];
                inc[n + i] = (u * s - c->norm_mean[1]) / c->norm_std[1];
                inc[2 * n + i] = (v * s - c->norm_mean[2]) / c->norm_std[2];
            }
        }
        memcpy(x, inc, sizeof(double) * len);
        pk_f64(x, c, n, &p, &k);
        energy = p + k;
        if (energies) energies[t] = energy;
        double viol = (energy - prev * (double)c->energy_r_max) / prev;
        if (viol > max_violation) max_violation = viol;
        if (traj) memcpy(traj + (size_t)t * len, x, sizeof(double) * len);
    }
    if (final_state) memcpy(final_state, x, sizeof(double) * len);
    free(x);
    free(inc);
    return max_violation;
}
