// A forward pass that allocates nothing, for callers that cannot call
// cudaMalloc when they run the model: host applications whose own pool
// allocator reserved the whole device up front (an extra cudaMalloc fails or
// fragments the pool), and plugins that work only in the buffers their host
// hands them.
//
// All intermediate buffers of the FP32 forward (the same kernels as
// jc_forward_device) live in one file-scope device array of kNoAllocBytes.
// Every GPU that loads this library holds that array until the process exits.
// The model's weights were allocated when the model was created; this call
// itself allocates no device or host memory. It runs the FP32 kernels for a
// model of either precision (a BF16 model keeps its f32 weights too).
#include <mutex>
#include <string>

#include "runtime.hpp"

namespace jc {

constexpr size_t kNoAllocBytes = 12u << 20;  // 12 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch on each device. Host code must not use
// the symbol itself as an address: on the host it names a host-side stand-in.
static void* g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

static unsigned char* scratch_for_current_device() {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) throw Error(JC_LIMIT, "device index out of range for the no-alloc scratch");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
        g_scratch_addr[dev] = p;
    }
    return static_cast<unsigned char*>(g_scratch_addr[dev]);
}

// Writes the instance descriptor (passed by value, so nothing on the host
// has to outlive the launch) into the scratch array.
__global__ void noalloc_put_instance(InstDev v, InstDev* dst) { *dst = v; }

void forward_noalloc(const Model& m, const float* d_state, const float* d_meta, float* d_inc, cudaStream_t s) {
    if (!d_state || !d_meta || !d_inc) throw Error(JC_BAD_ARGUMENT, "null buffer");
    const Dims& d = m.dims;
    const int tx = m.cfg.nx / m.cfg.patch, ty = m.cfg.ny / m.cfg.patch;
    const size_t R = (size_t)tx * ty, NC = (size_t)m.cfg.nx * m.cfg.ny;
    // carve the scratch: every buffer starts on a 256-byte boundary
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) / 256 * 256;
        return o;
    };
    const size_t o_inst = take(sizeof(InstDev));
    const size_t o_x = take(R * d.D * 4), o_qkv = take(R * 3 * d.D * 4), o_attn = take(R * d.D * 4);
    const size_t o_ff1 = take(R * d.F * 4), o_xn = take(R * d.D * 4), o_t1 = take(R * d.D * 4);
    const size_t o_z0 = take(R * d.HD * 4), o_zc = take(NC * kZcStride * 4), o_c1 = take(NC * d.HD * 4);
    if (off > kNoAllocBytes)
        throw Error(JC_LIMIT, "this grid needs " + std::to_string(off) + " bytes of scratch; the no-alloc forward holds " +
                                  std::to_string(kNoAllocBytes) + " bytes (12 MiB)");
    unsigned char* base = scratch_for_current_device();
    Pack p{};
    p.n_inst = 1;
    p.R = (int)R;
    p.NC = (long long)NC;
    p.n_tiles = cell_tiles(m.cfg.nx, m.cfg.ny);
    p.inst = reinterpret_cast<InstDev*>(base + o_inst);
    p.x = reinterpret_cast<float*>(base + o_x);
    p.qkv = reinterpret_cast<float*>(base + o_qkv);
    p.attn = reinterpret_cast<float*>(base + o_attn);
    p.ff1 = reinterpret_cast<float*>(base + o_ff1);
    p.xn = reinterpret_cast<float*>(base + o_xn);
    p.t1 = reinterpret_cast<float*>(base + o_t1);
    p.z0 = reinterpret_cast<float*>(base + o_z0);
    p.zc = reinterpret_cast<float*>(base + o_zc);
    p.c1 = reinterpret_cast<float*>(base + o_c1);
    InstDev inst{};
    inst.row0 = 0;
    inst.tx = tx;
    inst.ty = ty;
    inst.nx = m.cfg.nx;
    inst.ny = m.cfg.ny;
    inst.cell0 = 0;
    inst.state = const_cast<float*>(d_state);
    inst.out = d_inc;
    inst.pos = m.w.pos;
    inst.meta = d_meta;
    noalloc_put_instance<<<1, 1, 0, s>>>(inst, p.inst);
    cuda_check(cudaGetLastError(), "no-alloc descriptor");
    forward_f32(d, m.w.f32, p, kWriteIncrement, s);
}

}  // namespace jc
