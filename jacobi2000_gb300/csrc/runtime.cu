// Host runtime: checkpoint parsing (crates/engine/src/weights.rs,
// config.rs), device weight layouts, launch workspaces, the tick loop
// (crates/engine-cli/src/eval.rs:144-157) captured as CUDA graphs, and the
// batch runner.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
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
    if (c.dim % 4 || c.dim / c.heads > 64) throw Error(JC_LIMIT, "dim must be a multiple of 4 and dim/heads <= 64");
    if (c.layers <= 0 || c.layers > kMaxLayers) throw Error(JC_LIMIT, "layers must be in [1, 32]");
    if (c.meta_dim <= 0 || c.meta_dim > 64) throw Error(JC_LIMIT, "meta_dim must be in [1, 64]");
    if (c.mask_kind == 1 && (c.mask_radius < 0 || c.mask_dilation < 1))
        throw Error(JC_BAD_CHECKPOINT, "stencil radius must be >= 0 and dilation >= 1");
    c.head_dim = (int32_t)get(t, "head.to_cells.weight").shape.at(0);
    c.ff_inner = (int32_t)get(t, "blocks.0.ff1.weight").shape.at(1);
    if (c.head_dim % 4 || c.head_dim + c.channels > kZcStride)
        throw Error(JC_LIMIT, "cell-head width must be a multiple of 4 and at most 33");
    if (c.ff_inner % 4) throw Error(JC_LIMIT, "the MLP width must be a multiple of 4");

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
    cuda_check(cudaMalloc(&p, bytes ? (bytes + 255) / 256 * 256 : 256), "cudaMalloc", JC_OVER_BUDGET);
    ptrs.push_back(p);
    return p;
}

// Provisional addresses of image arrays start here until end_image() rebases
// them (never dereferenced: every slot is rebased, and counted, first).
static constexpr uint64_t kImageProvisional = 1ull << 52;

float* DeviceArena::upload(const std::vector<float>& v) {
    return static_cast<float*>(const_cast<void*>(upload_bytes(v.data(), v.size() * sizeof(float))));
}

const void* DeviceArena::upload_bytes(const void* src, size_t bytes) {
    if (imaging_) {
        const size_t off = (image.size() + 255) / 256 * 256;
        image.resize(off + (bytes ? bytes : 1), 0);
        if (bytes) std::memcpy(image.data() + off, src, bytes);
        image_arrays_++;
        return reinterpret_cast<const void*>(kImageProvisional + off);
    }
    void* d = alloc(bytes);
    cuda_check(cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice), "upload weights", JC_MAP);
    return d;
}

void DeviceArena::begin_image() {
    image.clear();
    image_arrays_ = 0;
    imaging_ = true;
}

std::vector<uint64_t> DeviceArena::end_image(const std::vector<const void**>& slots) {
    imaging_ = false;
    const uint64_t lo = kImageProvisional, hi = kImageProvisional + image.size();
    size_t provisional = 0;
    for (const void** sl : slots) {
        const uint64_t a = (uint64_t)(uintptr_t)*sl;
        if (a >= lo && a < hi) provisional++;
    }
    if (provisional != image_arrays_ || slots.size() != image_arrays_)
        throw Error(JC_CUDA_ERROR, "internal: the weight slots do not match the weight image");
    image_len = image.size();
    image_base = alloc(image_len);
    cuda_check(cudaMemcpy(image_base, image.data(), image_len, cudaMemcpyHostToDevice), "upload weights", JC_MAP);
    std::vector<uint64_t> off(slots.size());
    for (size_t i = 0; i < slots.size(); i++) {
        off[i] = (uint64_t)(uintptr_t)*slots[i] - lo;
        *slots[i] = static_cast<const char*>(image_base) + off[i];
    }
    image.clear();
    image.shrink_to_fit();
    return off;
}

void DeviceArena::release(void* p) {
    auto it = std::find(ptrs.begin(), ptrs.end(), p);
    if (it != ptrs.end()) {
        cudaFree(p);
        ptrs.erase(it);
    }
}

DeviceArena::~DeviceArena() {
    for (void* p : ptrs) cudaFree(p);
}

int cell_tiles(int nx, int ny) {
    return ((nx + kCellTile - 1) / kCellTile) * ((ny + kCellTile - 1) / kCellTile);
}

int conv_tiles(int w, int h) { return ((w + kConvTX - 1) / kConvTX) * ((h + kConvTY - 1) / kConvTY); }

void Workspace::alloc(DeviceArena& a, const Dims& d, int rows, long long cells, int inst, const BF16Path* bf) {
    max_rows = rows;
    max_cells = cells;
    max_inst = inst;
    Pack& p = base;
    p = Pack{};
    const size_t R = (size_t)rows, NC = (size_t)cells;
    p.inst = a.alloc_n<InstDev>(inst);
    p.proj = a.alloc_n<ProjSlot>(inst);
    p.x = a.alloc_n<float>(R * d.D);
    p.z0 = a.alloc_n<float>(R * d.HD);
    p.err = a.alloc_n<int>(1);
    cuda_check(cudaMemset(p.err, 0, sizeof(int)), "cudaMemset");
    if (bf) {
        bf->alloc_workspace(a, d, p, rows, cells, inst);
    } else {
        p.qkv = a.alloc_n<float>(R * 3 * d.D);
        p.attn = a.alloc_n<float>(R * d.D);
        p.ff1 = a.alloc_n<float>(R * d.F);
        p.xn = a.alloc_n<float>(R * d.D);
        p.t1 = a.alloc_n<float>(R * d.D);
        p.zc = a.alloc_n<float>(NC * kZcStride);
        p.c1 = a.alloc_n<float>(NC * d.HD);
    }
    states = a.alloc_n<float>(3 * NC);
    metas = a.alloc_n<float>((size_t)inst * 64);
}

void check_wait_flag(int* flag, cudaStream_t s) {
    int e = 0;
    cuda_check(cudaMemcpyAsync(&e, flag, sizeof(int), cudaMemcpyDeviceToHost, s), "error flag", JC_MAP);
    cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    if (e) {
        cudaMemsetAsync(flag, 0, sizeof(int), s);
        cudaStreamSynchronize(s);
        throw Error(JC_DEVICE_TIMEOUT, "a device-side wait exceeded its time limit; results of this call are invalid");
    }
}

void Workspace::check_timeout(cudaStream_t s) const { check_wait_flag(base.err, s); }

Pack Workspace::view(const Dims& d, int inst_base, int n, int row_base, int rows, long long cell_base,
                     long long cells, int tiles, int ttiles, int ctiles) const {
    Pack p = base;
    auto off = [](float* q, size_t o) { return q ? q + o : q; };
    p.n_inst = n;
    p.R = rows;
    p.NC = cells;
    p.n_tiles = tiles;
    p.n_ttiles = ttiles;
    p.n_ctiles = ctiles;
    if (base.tmaps) p.tmaps = static_cast<char*>(base.tmaps) + (size_t)inst_base * kMapsPerInst * 128;
    p.inst = base.inst + inst_base;
    p.proj = base.proj + inst_base;
    const size_t r = (size_t)row_base, c = (size_t)cell_base;
    p.x = off(base.x, r * d.D);
    p.qkv = off(base.qkv, r * 3 * d.D);
    p.attn = off(base.attn, r * d.D);
    p.ff1 = off(base.ff1, r * d.F);
    p.xn = off(base.xn, r * d.D);
    p.t1 = off(base.t1, r * d.D);
    p.z0 = off(base.z0, r * d.HD);
    p.zc = off(base.zc, c * kZcStride);
    p.c1 = off(base.c1, c * d.HD);
    for (int i = 0; i < Pack::kTokBufs; i++)
        if (base.bt[i]) p.bt[i] = base.bt[i] + r * base.bt_stride[i];
    for (int i = 0; i < Pack::kCellBufs; i++)
        if (base.bc[i]) p.bc[i] = base.bc[i] + c * base.bc_stride[i];
    return p;
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

static uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

static Dims dims_of(const jc_config& cfg) {
    Dims d{};
    d.D = cfg.dim;
    d.L = cfg.layers;
    d.heads = cfg.heads;
    d.F = cfg.ff_inner;
    d.HD = cfg.head_dim;
    d.C = cfg.channels;
    d.P = cfg.patch;
    d.meta_dim = cfg.meta_dim;
    d.mask_kind = cfg.mask_kind;
    d.radius = cfg.mask_radius;
    d.dilation = cfg.mask_dilation;
    for (int i = 0; i < 3; i++) {
        d.norm_mean[i] = cfg.norm_mean[i];
        d.norm_std[i] = cfg.norm_std[i];
    }
    d.norm_depth = cfg.norm_depth;
    d.g = cfg.g;
    d.energy_r_max = cfg.energy_r_max;
    return d;
}

static void upload_weights(const TensorMap& t, const Dims& dims, DeviceArena& arena, DeviceWeights& w) {
    const int D = dims.D, HD = dims.HD, C = dims.C;
    WeightsF32& f = w.f32;
    auto up = [&](const std::string& n) { return arena.upload(get(t, n).data); };
    f.embed_w = up("embed.weight");
    f.embed_b = up("embed.bias");
    f.meta_w = up("meta.weight");
    f.meta_b = up("meta.bias");
    w.pos = up("pos");
    for (int l = 0; l < dims.L; l++) {
        std::string p = "blocks." + std::to_string(l) + ".";
        auto& B = f.blk[l];
        B.n1g = up(p + "norm1.gamma");
        B.n1b = up(p + "norm1.beta");
        // q, k, v concatenated along the output axis, one [D, 3D] matrix
        // (the fused q/k/v of crates/engine/src/gpu.rs:288-301)
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
        B.wp = up(p + "proj.weight");
        B.bp = up(p + "proj.bias");
        B.n2g = up(p + "norm2.gamma");
        B.n2b = up(p + "norm2.beta");
        B.w1 = up(p + "ff1.weight");
        B.b1 = up(p + "ff1.bias");
        B.w2 = up(p + "ff2.weight");
        B.b2 = up(p + "ff2.bias");
    }
    f.norm_g = up("norm.gamma");
    f.norm_b = up("norm.beta");
    {
        // token_mix [co][ci][ky][kx] -> [(ky*3+kx)*D + ci][co]
        const auto& src = get(t, "head.token_mix.weight").data;
        std::vector<float> r((size_t)9 * D * D);
        for (int co = 0; co < D; co++)
            for (int ci = 0; ci < D; ci++)
                for (int k = 0; k < 9; k++) r[((size_t)k * D + ci) * D + co] = src[((size_t)co * D + ci) * 9 + k];
        f.tm_w = arena.upload(r);
        f.tm_b = up("head.token_mix.bias");
    }
    {
        const auto& src = get(t, "head.to_cells.weight").data;  // [HD][D][1][1] -> [D][HD]
        std::vector<float> r((size_t)D * HD);
        for (int co = 0; co < HD; co++)
            for (int ci = 0; ci < D; ci++) r[(size_t)ci * HD + co] = src[(size_t)co * D + ci];
        f.tc_w = arena.upload(r);
        f.tc_b = up("head.to_cells.bias");
    }
    {
        // conv1 [HD][HD+C][3][3] -> [(tap*kZcStride + ci)][HD], zero rows for the pad channel
        const auto& src = get(t, "head.conv1.weight").data;
        const int cin = HD + C;
        std::vector<float> r((size_t)9 * kZcStride * HD, 0.0f);
        for (int co = 0; co < HD; co++)
            for (int ci = 0; ci < cin; ci++)
                for (int k = 0; k < 9; k++)
                    r[((size_t)k * kZcStride + ci) * HD + co] = src[((size_t)co * cin + ci) * 9 + k];
        f.c1_w = arena.upload(r);
        f.c1_b = up("head.conv1.bias");
    }
    f.c2_w = up("head.conv2.weight");
    f.c2_b = up("head.conv2.bias");
    if (C == 3 && HD == 32) {
        const auto &src = get(t, "head.conv2.weight").data, &bias = get(t, "head.conv2.bias").data;
        w.conv2.reset(new Conv2Params());
        for (int co = 0; co < C; co++) {
            w.conv2->b[co] = bias[co];
            for (int ci = 0; ci < HD; ci++)
                for (int k = 0; k < 9; k++) w.conv2->w[(ci * 9 + k) * 3 + co] = src[((size_t)co * HD + ci) * 9 + k];
        }
        f.c2p = w.conv2.get();
    }
    uint64_t h = 1469598103934665603ull;
    for (auto& kv : t) {
        if (kv.first == "pos") continue;
        h = fnv1a(h, kv.first.data(), kv.first.size());
        h = fnv1a(h, kv.second.data.data(), kv.second.data.size() * 4);
    }
    w.shared_hash = h;
}

// Addresses of every device weight pointer of a model, in a fixed order (the
// order of the pre-packed image's slot table).
static std::vector<const void**> weight_slots(DeviceWeights& w, const Dims& d) {
    std::vector<const void**> s;
    WeightsF32& f = w.f32;
    auto add = [&](const float* const& p) { s.push_back(reinterpret_cast<const void**>(const_cast<const float**>(&p))); };
    add(f.embed_w);
    add(f.embed_b);
    add(f.meta_w);
    add(f.meta_b);
    add(w.pos);
    for (int l = 0; l < d.L; l++) {
        auto& B = f.blk[l];
        for (const float* const* p : {&B.n1g, &B.n1b, &B.wqkv, &B.bqkv, &B.wp, &B.bp, &B.n2g, &B.n2b, &B.w1, &B.b1,
                                      &B.w2, &B.b2})
            add(*p);
    }
    for (const float* const* p : {&f.norm_g, &f.norm_b, &f.tm_w, &f.tm_b, &f.tc_w, &f.tc_b, &f.c1_w, &f.c1_b,
                                  &f.c2_w, &f.c2_b})
        add(*p);
    if (w.bf16) w.bf16->weight_slots(s);
    return s;
}

uint64_t source_hash(const uint8_t* st, size_t st_len, const char* config_json) {
    uint64_t h = 1469598103934665603ull;
    h = fnv1a(h, st, st_len);
    if (config_json) h = fnv1a(h, config_json, std::strlen(config_json));
    return h;
}

// ---------------------------------------------------------------------------
// Pre-packed checkpoint: "JCPACK01", then little-endian u32 version (2),
// u32 precision, u64 source hash, u64 shared-tensor hash, the jc_config
// struct, u32 has-conv2 + the Conv2Params struct, u32 slot count + u64
// offsets, u64 image length, the image. Host and device are little-endian
// on every supported platform (x86-64 and aarch64).

static constexpr char kPackMagic[8] = {'J', 'C', 'P', 'A', 'C', 'K', '0', '1'};

namespace {
struct PackReader {
    const uint8_t* p;
    size_t n, at = 0;
    void get(void* dst, size_t k) {
        if (k > n - at) throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint is truncated");
        std::memcpy(dst, p + at, k);
        at += k;
    }
    template <class T>
    T get() {
        T v;
        get(&v, sizeof(T));
        return v;
    }
};
struct PackHeader {
    uint32_t precision = 0;
    uint64_t source = 0, shared = 0;
    jc_config cfg{};
    uint32_t has_conv2 = 0;
    Conv2Params conv2{};
    std::vector<uint64_t> slots;
    uint64_t image_len = 0;
    size_t image_at = 0;
};
PackHeader read_pack_header(const uint8_t* p, size_t n) {
    if (!p) throw Error(JC_BAD_ARGUMENT, "null pre-packed checkpoint");
    PackReader r{p, n};
    char magic[8];
    r.get(magic, 8);
    if (std::memcmp(magic, kPackMagic, 8) != 0) throw Error(JC_BAD_CHECKPOINT, "not a pre-packed checkpoint");
    if (r.get<uint32_t>() != 2) throw Error(JC_BAD_CHECKPOINT, "unsupported pre-packed checkpoint version");
    PackHeader h;
    h.precision = r.get<uint32_t>();
    h.source = r.get<uint64_t>();
    h.shared = r.get<uint64_t>();
    h.cfg = r.get<jc_config>();
    h.has_conv2 = r.get<uint32_t>();
    h.conv2 = r.get<Conv2Params>();
    const uint32_t ns = r.get<uint32_t>();
    if (ns > 100000) throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint: bad slot count");
    h.slots.resize(ns);
    for (auto& o : h.slots) o = r.get<uint64_t>();
    h.image_len = r.get<uint64_t>();
    if (h.image_len > n - r.at) throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint is truncated");
    h.image_at = r.at;
    for (uint64_t o : h.slots)
        if (o >= h.image_len || o % 256) throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint: bad slot offset");
    if (h.precision != JC_FP32 && h.precision != JC_BF16)
        throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint: bad precision");
    return h;
}
}  // namespace

uint64_t packed_source_hash(const uint8_t* packed, size_t len) { return read_pack_header(packed, len).source; }

// ---------------------------------------------------------------------------
// Model: one checkpoint, one grid, one request at a time.

Model::Model(const uint8_t* st, size_t st_len, const char* config_json, int prec) {
    if (prec != JC_FP32 && prec != JC_BF16) throw Error(JC_BAD_ARGUMENT, "precision must be JC_FP32 or JC_BF16");
    TensorMap t = parse_safetensors(st, st_len);
    cfg = parse_config(config_json, t);
    precision = prec;
    require_device();
    dims = dims_of(cfg);
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    source_hash = jc::source_hash(st, st_len, config_json);
    arena.begin_image();
    upload_weights(t, dims, arena, w);
    if (precision == JC_BF16) w.bf16 = std::make_unique<BF16Path>(dims, &t, &arena);
    slot_off_ = arena.end_image(weight_slots(w, dims));
    finish_init();
}

Model::Model(const uint8_t* packed, size_t len) {
    PackHeader h = read_pack_header(packed, len);
    cfg = h.cfg;
    precision = (int)h.precision;
    if (cfg.nx < 1 || cfg.ny < 1 || cfg.patch < 1 || cfg.nx % cfg.patch || cfg.ny % cfg.patch || cfg.layers < 0 ||
        cfg.layers > kMaxLayers || cfg.dim < 1 || cfg.heads < 1 || cfg.channels != 3)
        throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint: bad config");
    require_device();
    dims = dims_of(cfg);
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    source_hash = h.source;
    w.shared_hash = h.shared;
    if (h.has_conv2) {
        w.conv2.reset(new Conv2Params(h.conv2));
        w.f32.c2p = w.conv2.get();
    }
    if (precision == JC_BF16) w.bf16 = std::make_unique<BF16Path>(dims, nullptr, nullptr);
    std::vector<const void**> slots = weight_slots(w, dims);
    if (slots.size() != h.slots.size())
        throw Error(JC_BAD_CHECKPOINT, "pre-packed checkpoint: slot table does not match its config");
    arena.image_len = h.image_len;
    arena.image_base = arena.alloc(h.image_len);
    cuda_check(cudaMemcpy(arena.image_base, packed + h.image_at, h.image_len, cudaMemcpyHostToDevice),
               "upload weights", JC_MAP);
    for (size_t i = 0; i < slots.size(); i++) *slots[i] = static_cast<const char*>(arena.image_base) + h.slots[i];
    slot_off_ = h.slots;
    finish_init();
}

std::vector<uint8_t> Model::pack() const {
    std::vector<uint8_t> out;
    auto put = [&](const void* p, size_t k) {
        const uint8_t* b = static_cast<const uint8_t*>(p);
        out.insert(out.end(), b, b + k);
    };
    put(kPackMagic, 8);
    const uint32_t version = 2, prec = (uint32_t)precision, has_conv2 = w.conv2 ? 1u : 0u;
    put(&version, 4);
    put(&prec, 4);
    put(&source_hash, 8);
    put(&w.shared_hash, 8);
    put(&cfg, sizeof(cfg));
    put(&has_conv2, 4);
    Conv2Params c2{};
    if (w.conv2) c2 = *w.conv2;
    put(&c2, sizeof(c2));
    const uint32_t ns = (uint32_t)slot_off_.size();
    put(&ns, 4);
    put(slot_off_.data(), slot_off_.size() * 8);
    const uint64_t il = arena.image_len;
    put(&il, 8);
    const size_t at = out.size();
    out.resize(at + il);
    cuda_check(cudaMemcpy(out.data() + at, arena.image_base, il, cudaMemcpyDeviceToHost), "read weights", JC_MAP);
    return out;
}

void Model::finish_init() {
    const int tx = cfg.nx / cfg.patch, ty = cfg.ny / cfg.patch;
    const long long cells = (long long)cfg.nx * cfg.ny;
    state_len = (size_t)dims.C * cells;
    ws_.alloc(arena, dims, tx * ty, cells + 0, 1, w.bf16.get());
    pack_ = ws_.view(dims, 0, 1, 0, tx * ty, 0, cells, cell_tiles(cfg.nx, cfg.ny), conv_tiles(tx, ty),
                     conv_tiles(cfg.nx, cfg.ny));
    pack_.max_inst_cells = cells;
    inst_.row0 = 0;
    inst_.tx = tx;
    inst_.ty = ty;
    inst_.nx = cfg.nx;
    inst_.ny = cfg.ny;
    inst_.cell0 = 0;
    inst_.pos = w.pos;
    inst_.tile0 = 0;
    inst_.tt0 = 0;
    inst_.ct0 = 0;
    if (w.bf16) w.bf16->prepare(dims, pack_, &inst_, stream);
    d_inc_ = arena.alloc_n<float>(state_len);
    cuda_check(cudaMallocHost(&h_pinned_, (2 * state_len + 64) * sizeof(float)), "cudaMallocHost", JC_OVER_BUDGET);
}

Model::~Model() {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    if (h_pinned_) cudaFreeHost(h_pinned_);
}

void Model::meta_of(float* out) const {
    out[0] = std::log(cfg.dx);
    out[1] = std::log(cfg.dt);
    out[2] = std::log(cfg.g);
    out[3] = std::log(cfg.depth);
    out[4] = std::log(cfg.nu + 1e-6f);
}

void Model::forward_pack(const Pack& p, int mode, cudaStream_t s) const {
    if (precision == JC_BF16) w.bf16->forward(dims, w.f32, p, mode, s);
    else forward_f32(dims, w.f32, p, mode, s);
}

void Model::put_instance(float* state, float* out, const float* meta, uint32_t flags, cudaStream_t s) {
    InstDev i = inst_;
    i.state = state;
    i.out = out;
    i.meta = meta;
    i.flags = flags;
    // pageable source: the call returns once the bytes are staged
    cuda_check(cudaMemcpyAsync(pack_.inst, &i, sizeof(i), cudaMemcpyHostToDevice, s), "instance descriptor", JC_MAP);
}

void Model::forward_host(const float* state, const float* meta, float* inc) {
    if (!state || !meta || !inc) throw Error(JC_BAD_ARGUMENT, "null buffer");
    float* hs = h_pinned_;
    float* ho = h_pinned_ + state_len;
    float* hm = h_pinned_ + 2 * state_len;
    float* d_state = ws_.states;
    float* d_meta = ws_.metas;
    float* d_inc = d_inc_;
    std::memcpy(hs, state, state_len * 4);
    std::memcpy(hm, meta, cfg.meta_dim * 4);
    cuda_check(cudaMemcpyAsync(d_state, hs, state_len * 4, cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    cuda_check(cudaMemcpyAsync(d_meta, hm, cfg.meta_dim * 4, cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    put_instance(d_state, d_inc, d_meta, 0, stream);
    if (w.bf16) w.bf16->tune(dims, w.f32, pack_, stream);
    forward_pack(pack_, kWriteIncrement, stream);
    cuda_check(cudaMemcpyAsync(ho, d_inc, state_len * 4, cudaMemcpyDeviceToHost, stream), "D2H", JC_MAP);
    cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize", JC_POLL);
    ws_.check_timeout(stream);
    std::memcpy(inc, ho, state_len * 4);
}

void Model::step_host(const float* state, const float* meta, float* next) {
    forward_host(state, meta, next);
    for (size_t i = 0; i < state_len; i++) next[i] += state[i];  // cpu.rs:84-88
}

void Model::enqueue_rollout(int ticks, double* e, float* traj, cudaStream_t s) {
    projection(dims, pack_, 1, s);
    if (e) cuda_check(cudaMemcpyAsync(e, &pack_.proj[0].energy, 8, cudaMemcpyDeviceToDevice, s), "energy record");
    if (traj) cuda_check(cudaMemcpyAsync(traj, ws_.states, state_len * 4, cudaMemcpyDeviceToDevice, s), "traj");
    for (int t = 1; t <= ticks; t++) {
        forward_pack(pack_, kWriteNextState, s);
        projection(dims, pack_, 0, s);
        if (e)
            cuda_check(cudaMemcpyAsync(e + t, &pack_.proj[0].energy, 8, cudaMemcpyDeviceToDevice, s),
                       "energy record");
        if (traj)
            cuda_check(cudaMemcpyAsync(traj + (size_t)t * state_len, ws_.states, state_len * 4,
                                       cudaMemcpyDeviceToDevice, s),
                       "traj");
    }
}

cudaGraphExec_t Model::graph_for(const GraphKey& key, double* e, float* traj) {
    auto it = graphs_.find(key);
    if (it != graphs_.end()) return it->second;
    if (w.bf16) w.bf16->tune(dims, w.f32, pack_, key.s);
    cudaGraph_t g;
    cuda_check(cudaStreamBeginCapture(key.s, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
        enqueue_rollout(key.ticks, e, traj, key.s);
    } catch (...) {
        cudaStreamEndCapture(key.s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cuda_check(cudaStreamEndCapture(key.s, &g), "end capture");
    cudaGraphExec_t ge;
    cudaError_t err = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    cuda_check(err, "graph instantiate");
    graphs_.emplace(key, ge);
    return ge;
}

void Model::rollout_device(const float* d_x0, const float* d_meta_in, int ticks, uint32_t flags, float* d_final,
                           double* d_energies_out, cudaStream_t s) {
    if (ticks < 0) throw Error(JC_BAD_ARGUMENT, "ticks must be >= 0");
    if (flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown rollout flag");
    if (!s) s = stream;
    cuda_check(cudaMemcpyAsync(ws_.states, d_x0, state_len * 4, cudaMemcpyDeviceToDevice, s), "copy x0");
    cuda_check(cudaMemcpyAsync(ws_.metas, d_meta_in, cfg.meta_dim * 4, cudaMemcpyDeviceToDevice, s), "copy meta");
    put_instance(ws_.states, ws_.states, ws_.metas, flags, s);
    cuda_check(cudaGraphLaunch(graph_for(GraphKey{ticks, d_energies_out, nullptr, s, g_autotune.load()}, d_energies_out, nullptr), s),
               "graph launch");
    if (d_final)
        cuda_check(cudaMemcpyAsync(d_final, ws_.states, state_len * 4, cudaMemcpyDeviceToDevice, s), "copy final");
}

void Model::rollout_host(const float* x0, const float* meta, int ticks, uint32_t flags, float* final_state,
                         float* traj, double* energies) {
    if (!x0 || !meta || !final_state) throw Error(JC_BAD_ARGUMENT, "null buffer");
    if (ticks < 0) throw Error(JC_BAD_ARGUMENT, "ticks must be >= 0");
    if (flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown rollout flag");
    if (energies && ticks + 1 > energies_cap_) {
        if (d_energies_) arena.release(d_energies_);
        energies_cap_ = ticks + 1;
        d_energies_ = arena.alloc_n<double>((size_t)energies_cap_);
    }
    float* hs = h_pinned_;
    float* ho = h_pinned_ + state_len;
    float* hm = h_pinned_ + 2 * state_len;
    std::memcpy(hs, x0, state_len * 4);
    std::memcpy(hm, meta, cfg.meta_dim * 4);
    cuda_check(cudaMemcpyAsync(ws_.states, hs, state_len * 4, cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    cuda_check(cudaMemcpyAsync(ws_.metas, hm, cfg.meta_dim * 4, cudaMemcpyHostToDevice, stream), "H2D", JC_MAP);
    put_instance(ws_.states, ws_.states, ws_.metas, flags, stream);
    float* d_traj = traj ? arena.alloc_n<float>((size_t)(ticks + 1) * state_len) : nullptr;
    double* e = energies ? d_energies_ : nullptr;
    GraphKey key{ticks, e, d_traj, stream, g_autotune.load()};
    try {
        cuda_check(cudaGraphLaunch(graph_for(key, e, d_traj), stream), "graph launch");
        cuda_check(cudaMemcpyAsync(ho, ws_.states, state_len * 4, cudaMemcpyDeviceToHost, stream), "D2H", JC_MAP);
        if (energies)
            cuda_check(cudaMemcpyAsync(energies, d_energies_, (size_t)(ticks + 1) * 8, cudaMemcpyDeviceToHost, stream),
                       "D2H", JC_MAP);
        if (traj)
            cuda_check(cudaMemcpyAsync(traj, d_traj, (size_t)(ticks + 1) * state_len * 4, cudaMemcpyDeviceToHost,
                                       stream),
                       "D2H", JC_MAP);
        cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize", JC_POLL);
        ws_.check_timeout(stream);
    } catch (...) {
        if (d_traj) {
            auto it = graphs_.find(key);
            if (it != graphs_.end()) {
                cudaGraphExecDestroy(it->second);
                graphs_.erase(it);
            }
            arena.release(d_traj);
        }
        throw;
    }
    std::memcpy(final_state, ho, state_len * 4);
    if (d_traj) {
        // the trajectory buffer is per call: drop it and its graph
        auto it = graphs_.find(key);
        cudaGraphExecDestroy(it->second);
        graphs_.erase(it);
        arena.release(d_traj);
    }
}

void Model::forward_device(const float* d_state_in, const float* d_meta_in, float* d_inc_out, cudaStream_t s) {
    if (!d_state_in || !d_meta_in || !d_inc_out) throw Error(JC_BAD_ARGUMENT, "null buffer");
    if (!s) s = stream;
    put_instance(const_cast<float*>(d_state_in), d_inc_out, d_meta_in, 0, s);
    if (w.bf16) w.bf16->tune(dims, w.f32, pack_, s);
    forward_pack(pack_, kWriteIncrement, s);
}

std::map<std::string, std::pair<int, double>> Model::profile_forward(int iters) {
    KernelTimer kt;
    put_instance(ws_.states, d_inc_, ws_.metas, 0, stream);
    g_ktimer = &kt;
    try {
        for (int i = 0; i < iters; i++) forward_pack(pack_, kWriteIncrement, stream);
    } catch (...) {
        g_ktimer = nullptr;
        throw;
    }
    g_ktimer = nullptr;
    return kt.summary();
}

// ---------------------------------------------------------------------------
// Batch

Batch::Batch(jc_model* const* models, int n_models, int max_inst, long long max_cells) {
    if (!models || n_models <= 0) throw Error(JC_BAD_ARGUMENT, "a batch needs at least one model");
    if (max_inst <= 0 || max_cells <= 0) throw Error(JC_BAD_ARGUMENT, "max_instances and max_cells must be > 0");
    for (int i = 0; i < n_models; i++) {
        if (!models[i]) throw Error(JC_BAD_ARGUMENT, "null model in the list");
        models_.push_back(models[i]->m);
    }
    const Model& m0 = *models_[0];
    dims_ = m0.dims;
    precision_ = m0.precision;
    for (Model* m : models_) {
        const Dims& d = m->dims;
        bool same = d.D == dims_.D && d.L == dims_.L && d.heads == dims_.heads && d.F == dims_.F &&
                    d.HD == dims_.HD && d.C == dims_.C && d.P == dims_.P && d.meta_dim == dims_.meta_dim &&
                    d.mask_kind == dims_.mask_kind && d.radius == dims_.radius && d.dilation == dims_.dilation &&
                    d.norm_depth == dims_.norm_depth && d.g == dims_.g && d.energy_r_max == dims_.energy_r_max &&
                    m->precision == precision_;
        for (int i = 0; i < 3; i++)
            same = same && d.norm_mean[i] == dims_.norm_mean[i] && d.norm_std[i] == dims_.norm_std[i];
        if (!same)
            throw Error(JC_BAD_ARGUMENT,
                        "models of a batch must share hyper-parameters, mask, normalizer, g, energy_r_max and precision");
    }
    for (int i = 0; i < n_models; i++) {
        int g = i;
        for (int j = 0; j < i; j++)
            if (models_[j]->w.shared_hash == models_[i]->w.shared_hash) {
                g = group_of_[j];
                break;
            }
        group_of_.push_back(g);
    }
    const int pp = dims_.P * dims_.P;
    cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaStreamCreateWithFlags(&stream2_, cudaStreamNonBlocking), "cudaStreamCreate");
    ws_.alloc(arena_, dims_, (int)(max_cells / pp) + 1, max_cells, max_inst, m0.w.bf16.get());
    cuda_check(cudaMallocHost(&h_states_, 3 * (size_t)max_cells * 4), "cudaMallocHost", JC_OVER_BUDGET);
    cuda_check(cudaMallocHost(&h_metas_, (size_t)max_inst * 64 * 4), "cudaMallocHost", JC_OVER_BUDGET);
    cuda_check(cudaMallocHost(&h_slots_, (size_t)max_inst * sizeof(ProjSlot)), "cudaMallocHost", JC_OVER_BUDGET);
}

Batch::~Batch() {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
    if (stream2_) cudaStreamDestroy(stream2_);
    if (h_states_) cudaFreeHost(h_states_);
    if (h_metas_) cudaFreeHost(h_metas_);
    if (h_slots_) cudaFreeHost(h_slots_);
}

Batch::Plan Batch::plan(const jc_instance* in, int n) const {
    if (n < 0 || (n > 0 && !in)) throw Error(JC_BAD_ARGUMENT, "bad instance list");
    if (n > ws_.max_inst) throw Error(JC_OVER_BUDGET, "more instances than the batch was created for");
    Plan p;
    // group order: first appearance
    std::vector<int> gorder;
    for (int i = 0; i < n; i++) {
        const jc_instance& x = in[i];
        if (x.model < 0 || x.model >= (int)models_.size()) throw Error(JC_BAD_ARGUMENT, "instance model index out of range");
        if (x.ticks < 0) throw Error(JC_BAD_ARGUMENT, "instance ticks must be >= 0");
        if (x.flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown instance flag");
        if (!x.x0 || !x.meta || !x.final_state) throw Error(JC_BAD_ARGUMENT, "null instance buffer");
        if (x.reserved != 0) throw Error(JC_BAD_ARGUMENT, "jc_instance.reserved must be 0");
        if (x.task == JC_TASK_RECONSTRUCT) {
            if (x.reverse_model < 0 || x.reverse_model >= (int)models_.size())
                throw Error(JC_BAD_ARGUMENT, "reconstruct: reverse model index out of range");
            const Model &mf = *models_[x.model], &mr = *models_[x.reverse_model];
            if (mf.cfg.nx != mr.cfg.nx || mf.cfg.ny != mr.cfg.ny)
                throw Error(JC_BAD_ARGUMENT, "reconstruct: forward and reverse checkpoints differ in grid");
            if (!x.known || x.ticks < 1 || x.max_sweeps < 1)
                throw Error(JC_BAD_ARGUMENT, "reconstruct needs a known mask, ticks >= 1 and max_sweeps >= 1");
            continue;  // sweep phase, planned below
        }
        if (x.task != 0) throw Error(JC_BAD_ARGUMENT, "unknown instance task");
        int g = group_of_[x.model];
        if (std::find(gorder.begin(), gorder.end(), g) == gorder.end()) gorder.push_back(g);
    }
    int inst_base = 0, row_base = 0;
    long long cell_base = 0, state_off = 0;
    for (int g : gorder) {
        std::vector<int> idx;
        for (int i = 0; i < n; i++)
            if (in[i].task == 0 && group_of_[in[i].model] == g) idx.push_back(i);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return in[a].ticks > in[b].ticks; });
        Plan::Group G;
        G.model = g;
        G.inst_base = inst_base;
        G.n = (int)idx.size();
        G.row_base = row_base;
        G.cell_base = cell_base;
        G.cell_base_i = 0;
        G.max_cells = 0;
        int rows = 0, tiles = 0, ttiles = 0, ctiles = 0;
        long long cells = 0;
        for (int i : idx) {
            const Model& m = *models_[in[i].model];
            InstDev d{};
            d.row0 = rows;
            d.tx = m.cfg.nx / m.cfg.patch;
            d.ty = m.cfg.ny / m.cfg.patch;
            d.nx = m.cfg.nx;
            d.ny = m.cfg.ny;
            d.cell0 = cells;
            d.state = ws_.states + state_off;
            d.out = d.state;
            d.pos = m.w.pos;
            d.meta = ws_.metas + (size_t)(inst_base + (int)p.order.size() - G.inst_base) * 64;
            d.flags = in[i].flags;
            d.tile0 = tiles;
            d.tt0 = ttiles;
            d.ct0 = ctiles;
            p.inst.push_back(d);
            p.order.push_back(i);
            p.state_off.push_back(state_off);
            rows += d.tx * d.ty;
            cells += (long long)d.nx * d.ny;
            tiles += cell_tiles(d.nx, d.ny);
            ttiles += conv_tiles(d.tx, d.ty);
            ctiles += conv_tiles(d.nx, d.ny);
            state_off += 3LL * d.nx * d.ny;
            G.ticks.push_back(in[i].ticks);
            G.rows.push_back(rows);
            G.cells.push_back(cells);
            G.tiles.push_back(tiles);
            G.ttiles.push_back(ttiles);
            G.ctiles.push_back(ctiles);
            G.max_cells = std::max(G.max_cells, (long long)d.nx * d.ny);
            p.max_ticks = std::max(p.max_ticks, in[i].ticks);
        }
        inst_base += G.n;
        row_base += rows;
        cell_base += cells;
        if (row_base > ws_.max_rows || cell_base > ws_.max_cells)
            throw Error(JC_OVER_BUDGET, "the instances need more cells than the batch was created for");
        p.groups.push_back(std::move(G));
    }
    // meta slots follow the packed order
    for (size_t k = 0; k < p.inst.size(); k++) p.inst[k].meta = ws_.metas + k * 64;
    p.n_tick_inst = (int)p.inst.size();

    // reconstruct: one F sub-instance per t = 1..H (forward weights) and one
    // R sub-instance per t = 0..H-1 (reverse weights), grouped by weights
    struct Sub {
        const Model* m;
        size_t state_off, out_off;
        int recon;
    };
    std::map<int, std::vector<Sub>> subs;  // weight group -> sub-instances
    std::vector<int> sg_order;
    for (int i = 0; i < n; i++) {
        const jc_instance& x = in[i];
        if (x.task != JC_TASK_RECONSTRUCT) continue;
        const Model& mf = *models_[x.model];
        Plan::Recon r{};
        r.order = i;
        r.H = x.ticks;
        r.nx = mf.cfg.nx;
        r.ny = mf.cfg.ny;
        r.cells = (long long)r.nx * r.ny;
        r.max_sweeps = x.max_sweeps;
        r.tol = x.tol;
        const size_t len = 3 * (size_t)r.cells, H = (size_t)r.H;
        r.off_vol = p.recon_floats;
        p.recon_floats += (H + 1) * len;
        r.off_F = p.recon_floats;
        p.recon_floats += H * len;
        r.off_R = p.recon_floats;
        p.recon_floats += H * len;
        r.off_vals = p.recon_floats;
        p.recon_floats += (H + 1) * len;
        r.off_known = p.recon_bytes;
        p.recon_bytes += (H + 1) * (size_t)r.cells;
        const int gf = group_of_[x.model], gr = group_of_[x.reverse_model];
        for (int gg : {gf, gr})
            if (std::find(sg_order.begin(), sg_order.end(), gg) == sg_order.end()) sg_order.push_back(gg);
        const int ri = (int)p.recons.size();
        for (int t = 1; t <= r.H; t++)
            subs[gf].push_back({&mf, r.off_vol + (size_t)(t - 1) * len, r.off_F + (size_t)(t - 1) * len, ri});
        for (int t = 0; t < r.H; t++)
            subs[gr].push_back({models_[x.reverse_model], r.off_vol + (size_t)(t + 1) * len, r.off_R + (size_t)t * len, ri});
        p.recons.push_back(r);
    }
    int base = p.n_tick_inst;
    for (int g : sg_order) {
        Plan::Group G;
        G.model = g;
        G.inst_base = base;
        G.n = (int)subs[g].size();
        G.row_base = 0;
        G.cell_base = 0;
        G.cell_base_i = 0;
        G.max_cells = 0;
        int rows = 0, tiles = 0, ttiles = 0, ctiles = 0;
        long long cells = 0;
        for (auto& sb : subs[g]) {
            const Model& m = *sb.m;
            InstDev d{};
            d.row0 = rows;
            d.tx = m.cfg.nx / m.cfg.patch;
            d.ty = m.cfg.ny / m.cfg.patch;
            d.nx = m.cfg.nx;
            d.ny = m.cfg.ny;
            d.cell0 = cells;
            d.pos = m.w.pos;
            d.meta = ws_.metas + (size_t)(p.n_tick_inst + sb.recon) * 64;
            d.flags = 4u;
            d.tile0 = tiles;
            d.tt0 = ttiles;
            d.ct0 = ctiles;
            p.inst.push_back(d);
            p.sub_off.push_back({sb.state_off, sb.out_off});
            rows += d.tx * d.ty;
            cells += (long long)d.nx * d.ny;
            tiles += cell_tiles(d.nx, d.ny);
            ttiles += conv_tiles(d.tx, d.ty);
            ctiles += conv_tiles(d.nx, d.ny);
            G.rows.push_back(rows);
            G.cells.push_back(cells);
            G.tiles.push_back(tiles);
            G.ttiles.push_back(ttiles);
            G.ctiles.push_back(ctiles);
            G.ticks.push_back(0);
            G.max_cells = std::max(G.max_cells, (long long)d.nx * d.ny);
        }
        if (rows > ws_.max_rows || cells > ws_.max_cells)
            throw Error(JC_OVER_BUDGET, "a reconstruct sweep needs more cells than the batch was created for");
        base += G.n;
        p.sgroups.push_back(std::move(G));
    }
    if ((int)p.inst.size() > ws_.max_inst || p.n_tick_inst + (int)p.recons.size() > ws_.max_inst)
        throw Error(JC_OVER_BUDGET, "reconstruct sub-instances exceed the batch's instance capacity");
    return p;
}

void Batch::bind_recon(Plan& p) {
    if (p.recons.empty()) return;
    bool grew = false;
    if (p.recon_floats > recon_f_cap_) {
        if (recon_f_) arena_.release(recon_f_);
        recon_f_cap_ = p.recon_floats;
        recon_f_ = arena_.alloc_n<float>(recon_f_cap_);
        grew = true;
    }
    if (p.recon_bytes > recon_u8_cap_) {
        if (recon_u8_) arena_.release(recon_u8_);
        recon_u8_cap_ = p.recon_bytes;
        recon_u8_ = arena_.alloc_n<uint8_t>(recon_u8_cap_);
        grew = true;
    }
    if ((int)p.recons.size() > recon_cap_) {
        if (d_recon_) arena_.release(d_recon_);
        recon_cap_ = (int)p.recons.size();
        d_recon_ = arena_.alloc_n<ReconDev>(recon_cap_);
        grew = true;
    }
    if (grew) {  // cached graphs hold the old buffers
        for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
        graphs_.clear();
    }
    for (size_t k = 0; k < p.sub_off.size(); k++) {
        InstDev& d = p.inst[p.n_tick_inst + k];
        d.state = recon_f_ + p.sub_off[k].first;
        d.out = recon_f_ + p.sub_off[k].second;
    }
}

void Batch::enqueue_sweep(const Plan& p, cudaStream_t s) const {
    for (const auto& G : p.sgroups) {
        if (G.n == 0) continue;
        Pack v = ws_.view(dims_, G.inst_base, G.n, 0, G.rows.back(), 0, G.cells.back(), G.tiles.back(),
                          G.ttiles.back(), G.ctiles.back());
        v.max_inst_cells = G.max_cells;
        models_[G.model]->forward_pack(v, kWriteNextState, s);
    }
    long long mc = 0;
    int mh = 0;
    for (const auto& r : p.recons) {
        mc = std::max(mc, r.cells);
        mh = std::max(mh, r.H);
    }
    recon_update(d_recon_, (int)p.recons.size(), mc, mh, s);
}

void Batch::enqueue(const Plan& p, cudaStream_t s, bool capture) const {
    for (const auto& G : p.groups) {
        if (G.n == 0) continue;
        Pack v = ws_.view(dims_, G.inst_base, G.n, G.row_base, G.rows.back(), G.cell_base, G.cells.back(),
                          G.tiles.back(), G.ttiles.back(), G.ctiles.back());
        v.max_inst_cells = G.max_cells;
        projection(dims_, v, 1, s);
    }
    for (int t = 1; t <= p.max_ticks; t++) {
        for (const auto& G : p.groups) {
            int na = 0;
            while (na < G.n && G.ticks[na] >= t) na++;
            if (na == 0) continue;
            Pack v = ws_.view(dims_, G.inst_base, na, G.row_base, G.rows[na - 1], G.cell_base, G.cells[na - 1],
                              G.tiles[na - 1], G.ttiles[na - 1], G.ctiles[na - 1]);
            v.max_inst_cells = G.max_cells;
            models_[G.model]->forward_pack(v, kWriteNextState, s);
            projection(dims_, v, 0, s);
        }
        if (hook_) hook_->after_tick(t, s);
    }
    if (p.recons.empty()) return;
    const int nrec = (int)p.recons.size();
    {
        long long mc = 0;
        int mh = 0;
        for (const auto& r : p.recons) {
            mc = std::max(mc, r.cells);
            mh = std::max(mh, r.H);
        }
        recon_init(d_recon_, nrec, mc, mh, s);
    }
    if (!capture) {
        // outside a graph (profiling): sweeps up to the largest limit; frozen
        // instances are left unchanged by the update
        int most = 0;
        for (const auto& r : p.recons) most = std::max(most, r.max_sweeps);
        for (int k = 0; k < most; k++) {
            enqueue_sweep(p, s);
            recon_finalize(d_recon_, nrec, 0ull, 0, s);
        }
        return;
    }
    // a conditional while node: its body is one sweep plus the kernel that
    // decides on the device whether another sweep runs
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cuda_check(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &ndeps), "cudaStreamGetCaptureInfo");
    if (st != cudaStreamCaptureStatusActive) throw Error(JC_CUDA_ERROR, "reconstruct loop outside a capture");
    cudaGraphConditionalHandle h;
    cuda_check(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault), "conditional handle");
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cn;
    std::vector<cudaGraphNode_t> dv(deps, deps + ndeps);
    cuda_check(cudaGraphAddNode(&cn, g, dv.data(), nullptr, dv.size(), &cp), "conditional node");
    cuda_check(cudaStreamUpdateCaptureDependencies(s, &cn, nullptr, 1, cudaStreamSetCaptureDependencies),
               "capture dependencies");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cuda_check(cudaStreamBeginCaptureToGraph(stream2_, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
               "capture the loop body");
    try {
        enqueue_sweep(p, stream2_);
        recon_finalize(d_recon_, nrec, (unsigned long long)h, 1, stream2_);
    } catch (...) {
        cudaGraph_t tmp;
        cudaStreamEndCapture(stream2_, &tmp);
        throw;
    }
    cuda_check(cudaStreamEndCapture(stream2_, &body), "end body capture");
}

void Batch::upload_recon(const Plan& p, const jc_instance* in, bool device_ptrs, cudaStream_t s) {
    if (p.recons.empty()) return;
    const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    std::vector<ReconDev> rd;
    for (const auto& r : p.recons) {
        const jc_instance& x = in[r.order];
        const size_t len = 3 * (size_t)r.cells, H = (size_t)r.H;
        cuda_check(cudaMemcpyAsync(recon_f_ + r.off_vals, x.x0, (H + 1) * len * 4, kind, s), "reconstruct values",
                   JC_MAP);
        cuda_check(cudaMemcpyAsync(recon_u8_ + r.off_known, x.known, (H + 1) * (size_t)r.cells, kind, s),
                   "reconstruct mask", JC_MAP);
        ReconDev d{};
        d.vol = recon_f_ + r.off_vol;
        d.F = recon_f_ + r.off_F;
        d.R = recon_f_ + r.off_R;
        d.vals = recon_f_ + r.off_vals;
        d.known = recon_u8_ + r.off_known;
        d.cells = r.cells;
        d.H = r.H;
        d.max_sweeps = r.max_sweeps;
        d.tol = r.tol;
        rd.push_back(d);
    }
    cuda_check(cudaMemcpyAsync(d_recon_, rd.data(), rd.size() * sizeof(ReconDev), cudaMemcpyHostToDevice, s),
               "reconstruct descriptors", JC_MAP);
    // each reconstruct instance's meta, read by its sweep sub-instances
    for (size_t ri = 0; ri < p.recons.size(); ri++)
        cuda_check(cudaMemcpyAsync(ws_.metas + (size_t)(p.n_tick_inst + ri) * 64, in[p.recons[ri].order].meta,
                                   dims_.meta_dim * 4, kind, s),
                   "reconstruct meta", JC_MAP);
}

void Batch::rollout(const jc_instance* in, int n, bool device_ptrs, cudaStream_t s, TickHook* hook) {
    if (!s) s = stream_;
    Plan p = plan(in, n);
    if (n == 0) return;
    bind_recon(p);
    const int md = dims_.meta_dim;
    long long total = 0;
    for (size_t k = 0; k < p.order.size(); k++) {
        const jc_instance& x = in[p.order[k]];
        const InstDev& d = p.inst[k];
        size_t len = 3 * (size_t)d.nx * d.ny;
        if (device_ptrs) {
            cuda_check(cudaMemcpyAsync(ws_.states + p.state_off[k], x.x0, len * 4, cudaMemcpyDeviceToDevice, s),
                       "copy x0");
            cuda_check(cudaMemcpyAsync(ws_.metas + k * 64, x.meta, md * 4, cudaMemcpyDeviceToDevice, s), "copy meta");
        } else {
            std::memcpy(h_states_ + p.state_off[k], x.x0, len * 4);
            std::memcpy(h_metas_ + k * 64, x.meta, md * 4);
        }
        total = p.state_off[k] + (long long)len;
    }
    if (!device_ptrs) {
        cuda_check(cudaMemcpyAsync(ws_.states, h_states_, (size_t)total * 4, cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(ws_.metas, h_metas_, p.order.size() * 64 * 4, cudaMemcpyHostToDevice, s), "H2D",
                   JC_MAP);
    }
    cuda_check(cudaMemcpyAsync(ws_.base.inst, p.inst.data(), p.inst.size() * sizeof(InstDev), cudaMemcpyHostToDevice,
                               s),
               "instance descriptors", JC_MAP);
    upload_recon(p, in, device_ptrs, s);
    prepare_maps(p, s);
    std::vector<long long> key;
    key.push_back((long long)(uintptr_t)s);
    key.push_back(g_autotune.load());
    for (const auto& r : p.recons) {
        key.push_back(-1000000 - r.H);
        key.push_back(((long long)r.nx << 20) | r.ny);
        key.push_back((long long)in[r.order].model * 4096 + in[r.order].reverse_model);
    }
    for (const auto& G : p.groups) {
        key.push_back(-1 - G.model);
        for (size_t k = 0; k < G.ticks.size(); k++) {
            const InstDev& d = p.inst[G.inst_base + k];
            key.push_back(((long long)d.nx << 40) | ((long long)d.ny << 20) | G.ticks[k]);
            key.push_back((long long)(uintptr_t)d.pos);
        }
    }
    if (hook) {
        std::vector<float*> st(n, nullptr);
        for (size_t k = 0; k < p.order.size(); k++) st[p.order[k]] = ws_.states + p.state_off[k];
        hook->bind(st, s);
        key.push_back(-2000000000LL);
        key.push_back(hook->key());
    }
    auto it = graphs_.find(key);
    if (it == graphs_.end()) {
        cudaGraph_t g;
        cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
        hook_ = hook;
        try {
            enqueue(p, s, true);
        } catch (...) {
            hook_ = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        hook_ = nullptr;
        cuda_check(cudaStreamEndCapture(s, &g), "end capture");
        cudaGraphExec_t ge;
        cudaError_t err = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        cuda_check(err, "graph instantiate");
        it = graphs_.emplace(key, ge).first;
    }
    cuda_check(cudaGraphLaunch(it->second, s), "graph launch");
    std::vector<ReconDev> rres(p.recons.size());
    for (size_t ri = 0; ri < p.recons.size(); ri++) {
        const auto& r = p.recons[ri];
        const jc_instance& x = in[r.order];
        const size_t bytes = (size_t)(r.H + 1) * 3 * (size_t)r.cells * 4;
        cuda_check(cudaMemcpyAsync(x.final_state, recon_f_ + r.off_vol, bytes,
                                   device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s),
                   "reconstruct volume", JC_MAP);
    }
    if (!p.recons.empty())
        cuda_check(cudaMemcpyAsync(rres.data(), d_recon_, rres.size() * sizeof(ReconDev), cudaMemcpyDeviceToHost, s),
                   "reconstruct results", JC_MAP);
    if (device_ptrs) {
        for (size_t k = 0; k < p.order.size(); k++) {
            const InstDev& d = p.inst[k];
            cuda_check(cudaMemcpyAsync(in[p.order[k]].final_state, ws_.states + p.state_off[k],
                                       3 * (size_t)d.nx * d.ny * 4, cudaMemcpyDeviceToDevice, s),
                       "copy final");
        }
    } else {
        cuda_check(cudaMemcpyAsync(h_states_, ws_.states, (size_t)total * 4, cudaMemcpyDeviceToHost, s), "D2H",
                   JC_MAP);
    }
    cuda_check(cudaMemcpyAsync(h_slots_, ws_.base.proj, p.order.size() * sizeof(ProjSlot), cudaMemcpyDeviceToHost, s),
               "D2H", JC_MAP);
    cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    ws_.check_timeout(s);
    for (size_t k = 0; k < p.order.size(); k++) {
        const jc_instance& x = in[p.order[k]];
        const InstDev& d = p.inst[k];
        if (!device_ptrs) std::memcpy(x.final_state, h_states_ + p.state_off[k], 3 * (size_t)d.nx * d.ny * 4);
        if (x.energy) {
            x.energy[0] = h_slots_[k].energy;
            x.energy[1] = h_slots_[k].max_viol;
        }
    }
    for (size_t ri = 0; ri < p.recons.size(); ri++) {
        const jc_instance& x = in[p.recons[ri].order];
        if (x.energy) {
            x.energy[0] = rres[ri].sweeps;
            x.energy[1] = rres[ri].last_resid;
        }
    }
}

std::map<std::string, std::pair<int, double>> Batch::profile(const jc_instance* in, int n, bool device_ptrs) {
    Plan p = plan(in, n);
    bind_recon(p);
    cudaStream_t s = stream_;
    for (size_t k = 0; k < p.order.size(); k++) {
        const jc_instance& x = in[p.order[k]];
        const InstDev& d = p.inst[k];
        size_t len = 3 * (size_t)d.nx * d.ny;
        cuda_check(cudaMemcpyAsync(ws_.states + p.state_off[k], x.x0, len * 4,
                                   device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s),
                   "copy x0");
        cuda_check(cudaMemcpyAsync(ws_.metas + k * 64, x.meta, dims_.meta_dim * 4,
                                   device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s),
                   "copy meta");
    }
    cuda_check(cudaMemcpyAsync(ws_.base.inst, p.inst.data(), p.inst.size() * sizeof(InstDev), cudaMemcpyHostToDevice,
                               s),
               "instance descriptors", JC_MAP);
    upload_recon(p, in, device_ptrs, s);
    prepare_maps(p, s);
    KernelTimer kt;
    g_ktimer = &kt;
    try {
        enqueue(p, s, false);
    } catch (...) {
        g_ktimer = nullptr;
        throw;
    }
    g_ktimer = nullptr;
    auto out = kt.summary();
    ws_.check_timeout(s);
    return out;
}

void Batch::prepare_maps(const Plan& p, cudaStream_t s) const {
    const Model& m0 = *models_[0];
    if (!m0.w.bf16) return;
    for (const auto& G : p.groups) {
        if (G.n == 0) continue;
        Pack v = ws_.view(dims_, G.inst_base, G.n, G.row_base, G.rows.back(), G.cell_base, G.cells.back(),
                          G.tiles.back(), G.ttiles.back(), G.ctiles.back());
        m0.w.bf16->prepare(dims_, v, p.inst.data() + G.inst_base, s);
        m0.w.bf16->tune(dims_, m0.w.f32, v, s);
    }
    for (const auto& G : p.sgroups) {
        if (G.n == 0) continue;
        Pack v = ws_.view(dims_, G.inst_base, G.n, 0, G.rows.back(), 0, G.cells.back(), G.tiles.back(),
                          G.ttiles.back(), G.ctiles.back());
        m0.w.bf16->prepare(dims_, v, p.inst.data() + G.inst_base, s);
        m0.w.bf16->tune(dims_, m0.w.f32, v, s);
    }
}

}  // namespace jc
