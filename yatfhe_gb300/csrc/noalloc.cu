// noalloc.cu -- yg_pbs_noalloc: the full bootstrap without any allocation by the library.
//
// yg_pbs keeps the extracted ciphertexts between the blind-rotation and key-switching
// kernels in a buffer it takes from the stream-ordered allocator.  Some callers cannot
// let a library allocate device memory at all: applications whose device memory is
// handed out by their own allocator or budget and must not grow behind its back,
// serving paths that reserve everything at start-up and treat any later allocation as a
// fault, and embedders that forbid allocation calls after initialisation.  For them this
// entry point uses a fixed scratch array that is part of the loaded module instead.
//
// The scratch is kNoAllocScratchWords int32 words (16 MiB) in a file-scope __device__
// array: every GPU that loads the library holds it until the process exits.  One call
// handles at most kNoAllocScratchWords / (k N + 1) ciphertexts (4092 at N = 1024, 2046 at
// N = 2048); larger counts are rejected with YG_ERR_INVALID.
//
// The array's name is only a host-side stand-in in host code, so its device address is
// looked up with cudaGetSymbolAddress, once per device with that device current.  The
// driver loads a module's device variables lazily, so that lookup is also the moment the
// array's 16 MiB are committed on the device.  A call with count 0 does this set-up alone,
// and also loads the two kernels a call launches (kernels too are loaded on first use):
// make it at start-up, before any stream capture and before the point from which the
// caller allows no more allocation.  Without it, the first call with count > 0 on a device
// does the set-up itself.  All calls share the one array and it keeps the previous call's
// contents: the blind-rotation kernel overwrites every word the key switch then reads, so
// nothing has to start at zero, but calls that overlap on the GPU (on different streams, or
// from several threads without ordering) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.hpp"

namespace {

constexpr size_t kNoAllocScratchWords = (size_t)4 << 20;  // 16 MiB of int32
constexpr int kMaxDevices = 64;

__device__ __align__(256) int32_t g_noalloc_scratch[kNoAllocScratchWords];

std::mutex g_setup_mu;
int32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current); looked up once.
int32_t* scratch_on(int device) {
    if (device < 0 || device >= kMaxDevices) throw std::invalid_argument("device ordinal out of range");
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        yg::ck(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
        g_scratch_ptr[device] = static_cast<int32_t*>(p);
    }
    return g_scratch_ptr[device];
}

// The set-up a call with count 0 does on the context's device (current): the scratch
// address looked up, and the kernels of a call loaded in the context's launch shape.
void setup(const yg_ctx* ctx) {
    scratch_on(ctx->device);
    const int rc = yg::br_ctas_per_sm(ctx->logN, ctx->p.torus_bits, ctx->p.n, ctx->p.l_approx, ctx->per_cta,
                                      ctx->layout);
    if (rc == -1) yg::ck(cudaGetLastError(), "loading the blind-rotation kernel");
    if (!ctx->launch_set && ctx->latency_max > 0 &&
        yg::br_ctas_per_sm(ctx->logN, ctx->p.torus_bits, ctx->p.n, ctx->p.l_approx, 1, yg::kLayoutChannelCluster) == -1)
        yg::ck(cudaGetLastError(), "loading the blind-rotation kernel");  // a small batch's layout
    if (yg::preload_keyswitch() != 0) yg::ck(cudaGetLastError(), "loading the key-switching kernel");
}

}  // namespace

extern "C" size_t yg_pbs_noalloc_max_count(const yg_ctx* ctx) {
    if (!ctx) return 0;
    return kNoAllocScratchWords / ((size_t)ctx->p.k * ctx->p.N + 1);
}

extern "C" int yg_pbs_noalloc(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, int32_t* d_out, int count,
                              const int64_t* d_lut, void* stream) {
    if (int rc = yg::check_key(ctx, key, true, true)) return rc;
    if (count < 0 || (count > 0 && (!d_in || !d_out || !d_lut))) return yg::set_err(YG_ERR_INVALID, "bad buffers");
    if (count == 0)
        return yg::guarded([&] {
            yg::DeviceGuard g(ctx->device);
            setup(ctx);
            return YG_OK;
        });
    const size_t max_count = yg_pbs_noalloc_max_count(ctx);
    if ((size_t)count > max_count)
        return yg::set_err(YG_ERR_INVALID, "yg_pbs_noalloc: " + std::to_string(count) +
                                                " ciphertexts exceed the fixed scratch, at most " +
                                                std::to_string(max_count) + " per call at N = " +
                                                std::to_string(ctx->p.N));
    return yg::guarded([&] {
        yg::DeviceGuard g(ctx->device);
        int32_t* big = scratch_on(ctx->device);
        const int kN = ctx->p.k * ctx->p.N;
        yg::BrArgs a = yg::br_args(ctx, key, count);
        a.lwe_in = d_in;
        a.lut = d_lut;
        a.big_out = big;
        yg::check_launch(yg::launch_blind_rotate(ctx->logN, ctx->p.torus_bits, a, stream), "blind rotate launch");
        yg::KsArgs k{big, key->d_ksk, d_out, count, kN, ctx->p.n, ctx->p.ks_level, ctx->p.ks_radix_bits};
        yg::check_launch(yg::launch_keyswitch(k, stream), "keyswitch launch");
        return YG_OK;
    });
}
