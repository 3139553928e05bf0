// Host runtime: checkpoint parsing (crates/engine/src/weights.rs,
// config.rs), device weight layouts, the single-instance launch pack and the
// tick loop (crates/engine-cli/src/eval.rs:144-157) captured as CUDA graphs.
#include <cmath>
#include <cstring>
#include <string>

#include "bf16_path.hpp"
#include "json.hpp"
#include "runtime.hpp"

namespace jc {

void cuda_check(cudaError_t e, const char* what, jc_status code) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// ---------------------------------------------------------------------------
// safetensors (weights.rs:29-48)

TensorMap parse_safetensors(const uint8_t* p, size_t n) {
    if (!p || n < 8) throw Error(JC_BAD_CHECKPOINT, "safetensors: buffer shorter than the 8-byte header length");
    uint64_t hlen = 0;
    for (int i = 7; i >= 0; i--) hlen = (hlen << 8) | p[i];
    if (hlen > n - 8) throw Error(JC_BAD_CHECKPOINT, "safetensors: header length runs past the end of the buffer");
    Json h;
    try {
        h = Json::parse(reinterpret_cast<const char*>(p + 8), (size_t)hlen);
    } catch (const std::exception& e) {
        throw Error(JC_BAD_CHECKPOINT, std::string("safetensors header: ") + e.what());
    }
    if (h.kind != Json::Object) throw Error(JC_BAD_CHECKPOINT, "safetensors header is not a JSON object");
    const size_t start = 8 + (size_t)hlen;
    TensorMap out;
    for (auto& kv : h.obj) {
        const std::string& name = kv.first;
        if (name == "__metadata__") continue;
        try {
            const Json& v = kv.second;
            if (v.at("dtype").string() != "F32")
                throw Error(JC_BAD_CHECKPOINT, "tensor `" + name + "`: only F32 is supported");
            HostTensor t;
            size_t numel = 1;
            for (auto& s : v.at("shape").arr) {
                long long d = s.integer();
                if (d < 0) throw Error(JC_BAD_CHECKPOINT, "tensor `" + name + "`: negative dimension");
                t.shape.push_back(d);
                numel *= (size_t)d;
            }
            const Json& off = v.at("data_offsets");
            if (off.kind != Json::Array || off.arr.size() != 2)
                throw Error(JC_BAD_CHECKPOINT, "tensor `" + name + "`: bad data_offsets");
            long long a = off.arr[0].integer(), b = off.arr[1].integer();
            if (a < 0 || b < a || (size_t)(b - a) != numel * 4 || start + (size_t)b > n)
                throw Error(JC_BAD_CHECKPOINT, "tensor `" + name + "`: data_offsets do not match its shape or the buffer");
            t.data.resize(numel);
            std::memcpy(t.data.data(), p + start + a, numel * 4);  // little-endian hosts only
            out.emplace(name, std::move(t));
        } catch (const Error&) {
            throw;
        } catch (const std::exception& e) {
            throw Error(JC_BAD_CHECKPOINT, "tensor `" + name + "`: " + e.what());
        }
    }
    return out;
}

// ---------------------------------------------------------------------------
// config.json (config.rs:70-100)

static const HostTensor& get(const TensorMap& t, const std::string& name) {
    auto it = t.find(name);
    if (it == t.end()) throw Error(JC_BAD_CHECKPOINT, "missing tensor `" + name + "`");
    return it->second;
}

static void expect_shape(const TensorMap& t, const std::string& name, std::vector<int64_t> shape) {
    const HostTensor& x = get(t, name);
    if (x.shape != shape) {
        std::string s = "tensor `" + name + "` has shape [";
        for (size_t i = 0; i < x.shape.size(); i++) s += (i ? ", " : "") + std::to_string(x.shape[i]);
        s += "], expected [";
        for (size_t i = 0; i < shape.size(); i++) s += (i ? ", " : "") + std::to_string(shape[i]);
        throw Error(JC_BAD_SHAPE, s + "]");
    }
}

jc_config parse_config(const char* json, const TensorMap& t) {
    if (!json) throw Error(JC_BAD_ARGUMENT, "config_json is null");
    Json j;
    try {
        j = Json::parse(json, std::strlen(json));
    } catch (const std::exception& e) {
        throw Error(JC_BAD_CHECKPOINT, std::string("config.json: invalid JSON: ") + e.what());
    }
    jc_config c{};
    try {
        c.nx = (int32_t)j.at("nx").integer();
        c.ny = (int32_t)j.at("ny").integer();
        c.patch = (int32_t)j.at("patch").integer();
        c.channels = (int32_t)j.at("channels").integer();
        c.dim = (int32_t)j.at("dim").integer();
        c.layers = (int32_t)j.at("layers").integer();
        c.heads = (int32_t)j.at("heads").integer();
        c.meta_dim = (int32_t)j.at("meta_dim").integer();
        const Json& nrm = j.at("norm");
        const Json& mean = nrm.at("mean");
        const Json& stdv = nrm.at("std");
        if (mean.arr.size() != 3 || stdv.arr.size() != 3) throw std::runtime_error("norm.mean/std must have 3 entries");
        for (int i = 0; i < 3; i++) {
            c.norm_mean[i] = (float)mean.arr[i].number();
            c.norm_std[i] = (float)stdv.arr[i].number();
        }
        c.norm_depth = (float)nrm.at("depth").number();
        c.dx = (float)j.at("dx").number();
        c.dt = (float)j.at("dt").number();
        c.g = (float)j.at("g").number();
        c.depth = (float)j.at("depth").number();
        c.nu = (float)j.at("nu").number();
        const Json* r = j.find("energy_r_max");
        c.energy_r_max = (r && r->kind == Json::Number) ? (float)r->number() : 1.0f;
        const Json* m = j.find("mask");
        c.mask_kind = 0;
        c.mask_radius = 0;
        c.mask_dilation = 1;
        if (m && m->kind == Json::String) {
            if (m->str != "Full") throw std::runtime_error("unrecognized mask `" + m->str + "`");
        } else if (m && m->kind == Json::Object) {
            const Json& s = m->at("Stencil");
            c.mask_kind = 1;
            c.mask_radius = (int32_t)s.at("radius").integer();
            c.mask_dilation = (int32_t)s.at("dilation").integer();
        } else if (m && m->kind != Json::Null) {
            throw std::runtime_error("unrecognized mask");
        }
    } catch (const Error&) {
        throw;
    } catch (const std::exception& e) {
        throw Error(JC_BAD_CHECKPOINT, std::string("config.json: ") + e.what());
    }
    if (c.patch <= 0 || c.nx <= 0 || c.ny <= 0 || c.nx % c.patch || c.ny % c.patch)
        throw Error(JC_BAD_SHAPE, "grid " + std::to_string(c.nx) + "x" + std::to_string(c.ny) +
                                      " is not divisible by the patch size " + std::to_string(c.patch));
    if (c.channels != 3) throw Error(JC_BAD_SHAPE, "channels must be 3 (h, u, v)");
    if (c.dim <= 0 || c.heads <= 0 || c.dim % c.heads) throw Error(JC_BAD_SHAPE, "dim must be a multiple of heads");
    if (c.layers <= 0 || c.layers > kMaxLayers) throw Error(JC_LIMIT, "layers must be in [1, 32]");
    if (c.meta_dim <= 0 || c.meta_dim > 64) throw Error(JC_LIMIT, "meta_dim must be in [1, 64]");
    if (c.mask_kind == 1 && (c.mask_radius < 0 || c.mask_dilation < 1))
        throw Error(JC_BAD_CHECKPOINT, "stencil radius must be >= 0 and dilation >= 1");
    c.head_dim = (int32_t)get(t, "head.to_cells.weight").shape.at(0);
    c.ff_inner = (int32_t)get(t, "blocks.0.ff1.weight").shape.at(1);
    if (c.head_dim + c.channels > kZcStride) throw Error(JC_LIMIT, "cell-head width + channels must be <= 36");

    const int64_t D = c.dim, F = c.ff_inner, HD = c.head_dim, C = c.channels, P = c.patch;
    const int64_t T = (int64_t)(c.nx / P) * (c.ny / P);
    expect_shape(t, "embed.weight", {C * P * P, D});
    expect_shape(t, "embed.bias", {D});
    expect_shape(t, "meta.weight", {c.meta_dim, D});
    expect_shape(t, "meta.bias", {D});
    expect_shape(t, "pos", {1, T, D});
    for (int i = 0; i < c.layers; i++) {
        std::string p = "blocks." + std::to_string(i) + ".";
        for (const char* s : {"norm1.gamma", "norm1.beta", "norm2.gamma", "norm2.beta", "q.bias", "k.bias", "v.bias",
                              "proj.bias", "ff2.bias"})
            expect_shape(t, p + s, {D});
        for (const char* s : {"q.weight", "k.weight", "v.weight", "proj.weight"}) expect_shape(t, p + s, {D, D});
        expect_shape(t, p + "ff1.weight", {D, F});
        expect_shape(t, p + "ff1.bias", {F});
        expect_shape(t, p + "ff2.weight", {F, D});
    }
    expect_shape(t, "norm.gamma", {D});
    expect_shape(t, "norm.beta", {D});
    expect_shape(t, "head.token_mix.weight", {D, D, 3, 3});
    expect_shape(t, "head.token_mix.bias", {D});
    expect_shape(t, "head.to_cells.weight", {HD, D, 1, 1});
    expect_shape(t, "head.to_cells.bias", {HD});
    expect_shape(t, "head.conv1.weight", {HD, HD + C, 3, 3});
    expect_shape(t, "head.conv1.bias", {HD});
    expect_shape(t, "head.conv2.weight", {C, HD, 3, 3});
    expect_shape(t, "head.conv2.bias", {C});
    return c;
}

// ---------------------------------------------------------------------------

void* DeviceArena::alloc(size_t bytes) {
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, bytes ? bytes : 16), "cudaMalloc", JC_OVER_BUDGET);
    ptrs.push_back(p);
    return p;
}

float* DeviceArena::upload(const std::vector<float>& v) {
    float* d = alloc_n<float>(v.size());
    cuda_check(cudaMemcpy(d, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice), "upload weights", JC_MAP);
    return d;
}

DeviceArena::~DeviceArena() {
    for (void* p : ptrs) cudaFree(p);
}

static void require_device() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error(JC_NO_DEVICE, "no CUDA device");
    }
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice", JC_NO_DEVICE);
    cudaDeviceProp prop{};
    cuda_check(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties", JC_NO_DEVICE);
    if (prop.major != 10 || prop.minor != 3)
        throw Error(JC_NO_DEVICE, std::string("this library is built for sm_103 (GB300); device is ") + prop.name +
                                      " sm_" + std::to_string(prop.major) + std::to_string(prop.minor));
}

Model::Model(const uint8_t* st, size_t st_len, const char* config_json, int prec) {
    if (prec != JC_FP32 && prec != JC_BF16) throw Error(JC_BAD_ARGUMENT, "precision must be JC_FP32 or JC_BF16");
    TensorMap t = parse_safetensors(st, st_len);
    cfg = parse_config(config_json, t);
    precision = prec;
    require_device();

    dims.D = cfg.dim;
    dims.L = cfg.layers;
    dims.heads = cfg.heads;
    dims.F = cfg.ff_inner;
    dims.HD = cfg.head_dim;
    dims.C = cfg.channels;
    dims.P = cfg.patch;
    dims.meta_dim = cfg.meta_dim;
    dims.mask_kind = cfg.mask_kind;
    dims.radius = cfg.mask_radius;
    dims.dilation = cfg.mask_dilation;
    for (int i = 0; i < 3; i++) {
        dims.norm_mean[i] = cfg.norm_mean[i];
        dims.norm_std[i] = cfg.norm_std[i];
    }
    dims.norm_depth = cfg.norm_depth;
    dims.g = cfg.g;
    dims.energy_r_max = cfg.energy_r_max;

    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");

    const int D = dims.D, HD = dims.HD, C = dims.C;
    auto up = [&](const char* n) { return arena.upload(get(t, n).data); };
    wf32.embed_w = up("embed.weight");
    wf32.embed_b = up("embed.bias");
    wf32.meta_w = up("meta.weight");
    wf32.meta_b = up("meta.bias");
    d_pos = up("pos");
    for (int l = 0; l < dims.L; l++) {
        std::string p = "blocks." + std::to_string(l) + ".";
        auto& B = wf32.blk[l];
        B.n1g = up((p + "norm1.gamma").c_str());
        B.n1b = up((p + "norm1.beta").c_str());
        // q, k, v concatenated along the output axis, as one [D, 3D] matrix
        // (the fused q/k/v of crates/engine/src/gpu.rs:288-301).
        const auto &wq = get(t, p + "q.weight").data, &wk = get(t, p + "k.weight").data,
                   &wv = get(t, p + "v.weight").data;
        std::vector<float> wqkv((size_t)D * 3 * D), bqkv(3 * D);
        for (int r = 0; r < D; r++)
            for (int o = 0; o < D; o++) {
                wqkv[(size_t)r * 3 * D + o] = wq[(size_t)r * D + o];
                wqkv[(size_t)r * 3 * D + D + o] = wk[(size_t)r * D + o];
                wqkv[(size_t)r * 3 * D + 2 * D + o] = wv[(size_t)r * D + o];
            }
        for (int o = 0; o < D; o++) {
            bqkv[o] = get(t, p + "q.bias").data[o];
            bqkv[D + o] = get(t, p + "k.bias").data[o];
            bqkv[2 * D + o] = get(t, p + "v.bias").data[o];
        }
        B.wqkv = arena.upload(wqkv);
        B.bqkv = arena.upload(bqkv);
        B.wp = up((p + "proj.weight").c_str());
        B.bp = up((p + "proj.bias").c_str());
        B.n2g = up((p + "norm2.gamma").c_str());
        B.n2b = up((p + "norm2.beta").c_str());
        B.w1 = up((p + "ff1.weight").c_str());
        B.b1 = up((p + "ff1.bias").c_str());
        B.w2 = up((p + "ff2.weight").c_str());
        B.b2 = up((p + "ff2.bias").c_str());
    }
    wf32.norm_g = up("norm.gamma");
    wf32.norm_b = up("norm.beta");
    {
        // token_mix [co][ci][ky][kx] -> [(ky*3+kx)*D + ci][co]
        const auto& w = get(t, "head.token_mix.weight").data;
        std::vector<float> r((size_t)9 * D * D);
        for (int co = 0; co < D; co++)
            for (int ci = 0; ci < D; ci++)
                for (int k = 0; k < 9; k++) r[((size_t)k * D + ci) * D + co] = w[((size_t)co * D + ci) * 9 + k];
        wf32.tm_w = arena.upload(r);
        wf32.tm_b = up("head.token_mix.bias");
    }
    {
        const auto& w = get(t, "head.to_cells.weight").data;  // [HD][D][1][1] -> [D][HD]
        std::vector<float> r((size_t)D * HD);
        for (int co = 0; co < HD; co++)
            for (int ci = 0; ci < D; ci++) r[(size_t)ci * HD + co] = w[(size_t)co * D + ci];
        wf32.tc_w = arena.upload(r);
        wf32.tc_b = up("head.to_cells.bias");
    }
    {
        // conv1 [HD][HD+C][3][3] -> [(tap*kZcStride + ci)][HD], zero rows for the pad channel
        const auto& w = get(t, "head.conv1.weight").data;
        const int cin = HD + C;
        std::vector<float> r((size_t)9 * kZcStride * HD, 0.0f);
        for (int co = 0; co < HD; co++)
            for (int ci = 0; ci < cin; ci++)
                for (int k = 0; k < 9; k++) r[((size_t)k * kZcStride + ci) * HD + co] = w[((size_t)co * cin + ci) * 9 + k];
        wf32.c1_w = arena.upload(r);
        wf32.c1_b = up("head.conv1.bias");
    }
    wf32.c2_w = up("head.conv2.weight");
    wf32.c2_b = up("head.conv2.bias");

    if (precision == JC_BF16) bf16 = std::make_unique<BF16Path>(dims, t, arena);

    // single-instance pack over the model's own grid
    const int tx = cfg.nx / cfg.patch, ty = cfg.ny / cfg.patch;
    pack.n_inst = 1;
    pack.R = tx * ty;
    pack.NC = (long long)cfg.nx * cfg.ny;
    state_len = (size_t)C * cfg.nx * cfg.ny;
    alloc_pack_workspace(pack);
    d_state = arena.alloc_n<float>(state_len);
    d_inc = arena.alloc_n<float>(state_len);
    d_meta = arena.alloc_n<float>(64);
    host_inst.row0 = 0;
    host_inst.tx = tx;
    host_inst.ty = ty;
    host_inst.nx = cfg.nx;
    host_inst.ny = cfg.ny;
    host_inst.cell0 = 0;
    host_inst.pos = d_pos;
    host_inst.meta = d_meta;
    host_inst.proj = 0;
    {
        std::vector<int> zeros_r(pack.R, 0);
        cuda_check(cudaMemcpy(pack.row_inst, zeros_r.data(), zeros_r.size() * sizeof(int), cudaMemcpyHostToDevice),
                   "upload row table", JC_MAP);
        std::vector<int> zeros_c((size_t)pack.NC, 0);
        cuda_check(cudaMemcpy(pack.cell_inst, zeros_c.data(), zeros_c.size() * sizeof(int), cudaMemcpyHostToDevice),
                   "upload cell table", JC_MAP);
    }
    cuda_check(cudaMallocHost(&h_pinned, (2 * state_len + 64) * sizeof(float)), "cudaMallocHost", JC_OVER_BUDGET);
}

Model::~Model() {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    if (h_pinned) cudaFreeHost(h_pinned);
}

void Model::alloc_pack_workspace(Pack& p) {
    const size_t R = (size_t)p.R, NC = (size_t)p.NC;
    const int D = dims.D;
    p.inst = arena.alloc_n<InstDev>(p.n_inst);
    p.row_inst = arena.alloc_n<int>(R);
    p.cell_inst = arena.alloc_n<int>(NC);
    p.proj = arena.alloc_n<ProjSlot>(p.n_inst);
    p.x = arena.alloc_n<float>(R * D);
    p.qkv = arena.alloc_n<float>(R * 3 * D);
    p.attn = arena.alloc_n<float>(R * D);
    p.ff1 = arena.alloc_n<float>(R * dims.F);
    p.xn = arena.alloc_n<float>(R * D);
    p.t1 = arena.alloc_n<float>(R * D);
    p.z0 = arena.alloc_n<float>(R * dims.HD);
    p.zc = arena.alloc_n<float>(NC * kZcStride);
    p.c1 = arena.alloc_n<float>(NC * dims.HD);
}

void Model::set_single_instance(float* state, float* out, const float* meta) {
    InstDev i = host_inst;
    i.state = state;
    i.out = out;
    i.meta = meta;
    // pageable source: the call returns once the bytes are staged
    cuda_check(cudaMemcpyAsync(pack.inst, &i, sizeof(i), cudaMemcpyHostToDevice, stream), "instance descriptor",
               JC_MAP);
}

void Model::meta_of(float* out) const {
    out[0] = std::log(cfg.dx);
    out[1] = std::log(cfg.dt);
    out[2] = std::log(cfg.g);
    out[3] = std::log(cfg.depth);
    out[4] = std::log(cfg.nu + 1e-6f);
}

void Model::forward_pack(const Pack& p, int mode, cudaStream_t s) {
    if (precision == JC_BF16) bf16->forward(dims, wf32, p, mode, s);
    else forward_f32(dims, wf32, p, mode, s);
}

void Model::forward_host(const float* state, const float* meta, float* inc) {
    if (!state || !meta || !inc) throw Error(JC_BAD_ARGUMENT, "null buffer");
    float* hs = h_pinned;
    float* hm = h_pinned + 2 * state_len;
    std::memcpy(hs, state, state_len * sizeof(float));
    std::memcpy(hm, meta, cfg.meta_dim * sizeof(float));
    cuda_check(cudaMemcpyAsync(d_state, hs, state_len * sizeof(float), cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    cuda_check(cudaMemcpyAsync(d_meta, hm, cfg.meta_dim * sizeof(float), cudaMemcpyHostToDevice, stream), "H2D",
               JC_MAP);
    set_single_instance(d_state, d_inc, d_meta);
    forward_pack(pack, kWriteIncrement, stream);
    cuda_check(cudaMemcpyAsync(hs + state_len, d_inc, state_len * sizeof(float), cudaMemcpyDeviceToHost, stream),
               "D2H", JC_MAP);
    cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize", JC_POLL);
    std::memcpy(inc, hs + state_len, state_len * sizeof(float));
}

void Model::step_host(const float* state, const float* meta, float* next) {
    forward_host(state, meta, next);
    for (size_t i = 0; i < state_len; i++) next[i] += state[i];  // cpu.rs:84-88
}

void Model::enqueue_rollout(int ticks, uint32_t flags, double* d_energies_out, float* d_traj, cudaStream_t s) {
    projection(dims, pack, flags, 1, s);
    if (d_energies_out)
        cuda_check(cudaMemcpyAsync(d_energies_out, &pack.proj[0].energy, sizeof(double), cudaMemcpyDeviceToDevice, s),
                   "energy record");
    if (d_traj) cuda_check(cudaMemcpyAsync(d_traj, d_state, state_len * 4, cudaMemcpyDeviceToDevice, s), "traj");
    for (int t = 1; t <= ticks; t++) {
        forward_pack(pack, kWriteNextState, s);
        projection(dims, pack, flags, 0, s);
        if (d_energies_out)
            cuda_check(cudaMemcpyAsync(d_energies_out + t, &pack.proj[0].energy, sizeof(double),
                                       cudaMemcpyDeviceToDevice, s),
                       "energy record");
        if (d_traj)
            cuda_check(cudaMemcpyAsync(d_traj + (size_t)t * state_len, d_state, state_len * 4,
                                       cudaMemcpyDeviceToDevice, s),
                       "traj");
    }
}

void Model::rollout_device(const float* d_x0, const float* d_meta_in, int ticks, uint32_t flags, float* d_final,
                           double* d_energies_out, cudaStream_t s) {
    if (ticks < 0) throw Error(JC_BAD_ARGUMENT, "ticks must be >= 0");
    if (flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown rollout flag");
    if (!s) s = stream;
    if (d_x0 != d_state)
        cuda_check(cudaMemcpyAsync(d_state, d_x0, state_len * 4, cudaMemcpyDeviceToDevice, s), "copy x0");
    if (d_meta_in != d_meta)
        cuda_check(cudaMemcpyAsync(d_meta, d_meta_in, cfg.meta_dim * 4, cudaMemcpyDeviceToDevice, s), "copy meta");
    {
        InstDev i = host_inst;
        i.state = d_state;
        i.out = d_state;
        i.meta = d_meta;
        cuda_check(cudaMemcpyAsync(pack.inst, &i, sizeof(i), cudaMemcpyHostToDevice, s), "instance descriptor",
                   JC_MAP);
    }
    GraphKey key{ticks, flags, d_energies_out, nullptr, s};
    auto it = graphs_.find(key);
    if (it == graphs_.end()) {
        cudaGraph_t g;
        cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
        try {
            enqueue_rollout(ticks, flags, d_energies_out, nullptr, s);
        } catch (...) {
            cudaStreamEndCapture(s, &g);
            throw;
        }
        cuda_check(cudaStreamEndCapture(s, &g), "end capture");
        cudaGraphExec_t ge;
        cuda_check(cudaGraphInstantiate(&ge, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        it = graphs_.emplace(key, ge).first;
    }
    cuda_check(cudaGraphLaunch(it->second, s), "graph launch");
    if (d_final && d_final != d_state)
        cuda_check(cudaMemcpyAsync(d_final, d_state, state_len * 4, cudaMemcpyDeviceToDevice, s), "copy final");
}

void Model::rollout_host(const float* x0, const float* meta, int ticks, uint32_t flags, float* final_state,
                         float* traj, double* energies) {
    if (!x0 || !meta || !final_state) throw Error(JC_BAD_ARGUMENT, "null buffer");
    if (ticks < 0) throw Error(JC_BAD_ARGUMENT, "ticks must be >= 0");
    if (flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown rollout flag");
    if (energies && ticks + 1 > energies_cap) {
        energies_cap = ticks + 1;
        d_energies = arena.alloc_n<double>((size_t)energies_cap);
    }
    float* hs = h_pinned;
    float* hm = h_pinned + 2 * state_len;
    std::memcpy(hs, x0, state_len * 4);
    std::memcpy(hm, meta, cfg.meta_dim * 4);
    cuda_check(cudaMemcpyAsync(d_state, hs, state_len * 4, cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    cuda_check(cudaMemcpyAsync(d_meta, hm, cfg.meta_dim * 4, cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    {
        InstDev i = host_inst;
        i.state = d_state;
        i.out = d_state;
        i.meta = d_meta;
        cuda_check(cudaMemcpyAsync(pack.inst, &i, sizeof(i), cudaMemcpyHostToDevice, stream), "descriptor", JC_MAP);
    }
    float* d_traj = nullptr;
    if (traj) d_traj = arena.alloc_n<float>((size_t)(ticks + 1) * state_len);
    GraphKey key{ticks, flags, energies ? d_energies : nullptr, d_traj, stream};
    auto it = graphs_.find(key);
    if (it == graphs_.end()) {
        cudaGraph_t g;
        cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        try {
            enqueue_rollout(ticks, flags, energies ? d_energies : nullptr, d_traj, stream);
        } catch (...) {
            cudaStreamEndCapture(stream, &g);
            throw;
        }
        cuda_check(cudaStreamEndCapture(stream, &g), "end capture");
        cudaGraphExec_t ge;
        cuda_check(cudaGraphInstantiate(&ge, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        it = graphs_.emplace(key, ge).first;
    }
    cuda_check(cudaGraphLaunch(it->second, stream), "graph launch");
    cuda_check(cudaMemcpyAsync(hs + state_len, d_state, state_len * 4, cudaMemcpyDeviceToHost, stream), "D2H", JC_MAP);
    if (energies)
        cuda_check(cudaMemcpyAsync(energies, d_energies, (size_t)(ticks + 1) * 8, cudaMemcpyDeviceToHost, stream),
                   "D2H", JC_MAP);
    if (traj)
        cuda_check(cudaMemcpyAsync(traj, d_traj, (size_t)(ticks + 1) * state_len * 4, cudaMemcpyDeviceToHost, stream),
                   "D2H", JC_MAP);
    cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize", JC_POLL);
    std::memcpy(final_state, hs + state_len, state_len * 4);
    if (traj) {
        // drop the per-call trajectory buffer's graph (its pointer is not reused)
        cudaGraphExecDestroy(it->second);
        graphs_.erase(it);
        cudaFree(d_traj);
        arena.ptrs.pop_back();
    }
}

void Model::forward_device(const float* d_state_in, const float* d_meta_in, float* d_inc_out, cudaStream_t s) {
    if (!d_state_in || !d_meta_in || !d_inc_out) throw Error(JC_BAD_ARGUMENT, "null buffer");
    if (!s) s = stream;
    InstDev i = host_inst;
    i.state = const_cast<float*>(d_state_in);
    i.out = d_inc_out;
    i.meta = d_meta_in;
    cuda_check(cudaMemcpyAsync(pack.inst, &i, sizeof(i), cudaMemcpyHostToDevice, s), "descriptor", JC_MAP);
    forward_pack(pack, kWriteIncrement, s);
}

}  // namespace jc
