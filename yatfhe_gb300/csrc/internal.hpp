// internal.hpp -- definitions shared by the host-side translation units of the library
// (context and key objects, error reporting, launch-argument assembly).
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>

#include "../../include/yatfhe_gb300.h"
#include "pbs_kernels.cuh"

namespace yg {

struct QTables;

// Message of the last failure on this thread (yg_last_error).
std::string& last_error_slot();

inline int set_err(int code, const std::string& msg) {
    last_error_slot() = msg;
    return code;
}

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Runs f(), mapping exceptions to the ABI's status codes.
template <typename F>
int guarded(F&& f) {
    try {
        return f();
    } catch (const CudaError& e) {
        return set_err(YG_ERR_CUDA, e.what());
    } catch (const std::invalid_argument& e) {
        return set_err(YG_ERR_INVALID, e.what());
    } catch (const std::bad_alloc&) {
        return set_err(YG_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return set_err(YG_ERR_IO, e.what());
    }
}

// A kernel launcher's status: a CUDA error if one was raised, else an unsupported launch
// shape (e.g. more shared memory than an SM has); never silently nothing launched.
inline void check_launch(int rc, const char* what) {
    if (rc == 0) return;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
    throw std::invalid_argument(std::string(what) + ": launch shape not supported for these parameters");
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) ck(cudaSetDevice(dev), "cudaSetDevice");
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace yg

struct yg_ctx {
    yg_params p{};
    int logN = 0;
    int ps = 0;             // RNS prime set (rns.cuh), fixed by the torus width
    int device = 0;
    uint64_t q = 0;
    uint2* d_tw = nullptr;  // [3][3N]: forward twiddles (N), then the inverse table (2N) per channel
    uint2* d_tw16 = nullptr;  // [3][N]: psi^-e in natural order (16-residue inverse, T = 32 at N = 1024)
    yg::Chan ch[yg::kChannels]{};
    yg::Crt crt{};
    uint32_t conv_scale[yg::kChannels]{}, conv_scale_s[yg::kChannels]{};
    std::shared_ptr<yg::QTables> qtab;
    int sm_count = 0;
    int layout = 0;        // YG_LAYOUT_* of the blind rotation (yg_ctx_set_launch)
    int per_cta = 1;       // ciphertexts per blind-rotation CTA (yg_ctx_set_launch)
    int ctas_per_sm = 0;   // persistent CTAs per SM, 0 = one CTA per ciphertext group
    bool launch_set = false;  // yg_ctx_set_launch was called: its shape applies to every batch
    int latency_max = 0;      // batches of at most this many run in the channel-cluster layout
                              // while launch_set is false (0: that layout does not exist here)
    cudaStream_t side = nullptr;  // second stream of the pipelined host-buffer bootstrap
    std::mutex side_mu;           // creates `side` once
    uint64_t* d_qfwd = nullptr;   // [wf | wfp] (N each): mod-q forward twiddles, made by the first RLWE encryption
    std::mutex qfwd_mu;           // creates `d_qfwd` once
};

struct yg_key {
    yg_ctx* ctx = nullptr;
    uint32_t* d_bsk = nullptr;
    int32_t* d_ksk = nullptr;
    size_t bsk_bytes = 0, ksk_bytes = 0;
    // A lazy ("OURS") key instead of GINX rows: the half rows [n][L][2][N] in the torus word
    // size, and one block of [wi | wip | wf | wfp] (N each) + [s2 | s2p] ([Ls][2][N] each).
    void* d_lazy_cprime = nullptr;
    uint64_t* d_lazy_tab = nullptr;
    int lazy_ls = 0;
    bool lazy() const { return d_lazy_cprime != nullptr; }
    // A group-g key of the TrgswDft family: the used levels' words [keys][L][2][2][N], and one
    // block of [wi | wip | wf | wfp] (N each) + psi^j 2^64 mod q [2N] + slot exponents [N].
    uint64_t* d_group = nullptr;
    uint64_t* d_group_tab = nullptr;
    int group = 0, group_levels = 0;
    bool grouped() const { return d_group != nullptr; }
};

namespace yg {

// need_bsk: the key must hold GINX rows, or (lazy_ok) GINX rows, a lazy key or a group key.
int check_key(const yg_ctx* c, const yg_key* k, bool need_bsk, bool need_ksk, bool lazy_ok = false);

// Blind-rotation launch arguments of a context and key (buffers and count left empty).
BrArgs br_args(const yg_ctx* c, const yg_key* key);
// br_args for a batch of `count` GINX ciphertexts: the context's launch shape, or for a small
// batch on a context whose shape was never set the channel-cluster layout.
BrArgs br_args(const yg_ctx* c, const yg_key* key, int count);
// The same for a lazy key (the lazy blind rotation).
LazyBrArgs lazy_launch_args(const yg_ctx* c, const yg_key* key);
// A lazy key's device parts: the half rows (bytes), the table block of [wi | wip | wf | wfp]
// (N words each) then [s2 | s2p] ([Ls][k+1][N] each), and the kernel's view of one key.
size_t lazy_cprime_bytes(const yg_params& p);
size_t lazy_tab_words(const yg_params& p, int Ls);
LazyKeyRef lazy_key_ref(const yg_params& p, const void* cprime, const uint64_t* tab, int Ls);

}  // namespace yg
