// gdfjk_host.cu — host side of the GB300 DF-JK engine and its C ABI (include/gdfjk.h).
//
// One handle = one device, one CUDA stream, B resident in HBM in the tiled layout of
// common.cuh, and workspaces sized on first use.  A Fock build (gdfjk_compute) follows
// JK::compute (psi4/src/psi4/libfock/jk.cc:595-681) for one density:
//   compute_D (jk.cc:314-354)  ->  MemDFJK::compute_JK (MemDFJK.cc:97-111):
//   zero J/K, then DFHelper::compute_J_symm / compute_K (dfhelper.cc:3162-3377)
// with the J passes and the K kernels on the GPU.  Errors become status codes with a
// message (psi4 throws PSIEXCEPTION at the same places: jk.cc:607-634 for mismatched
// C_left/C_right, dfhelper.cc:167-173 for memory).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gdfjk.h"
#include "common.cuh"
#include "mixed.cuh"
#include "oz.cuh"

using namespace gdfjk;

namespace {
thread_local std::string g_create_err;
}

int gdfjk::report_error(int code, const std::string& msg) {
    g_create_err = msg;
    return code;
}

namespace {
// fault injection: let g_alloc_pass allocations through, then refuse g_alloc_refuse
std::mutex g_alloc_mutex;
long g_alloc_pass = 0, g_alloc_refuse = 0;
}  // namespace

bool gdfjk::alloc_refused() {
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    if (g_alloc_refuse <= 0) return false;
    if (g_alloc_pass > 0) {
        --g_alloc_pass;
        return false;
    }
    --g_alloc_refuse;
    return true;
}

cudaError_t gdfjk::engine_malloc(void** p, size_t bytes) {
    *p = nullptr;
    if (alloc_refused()) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

cudaError_t gdfjk::big_alloc(void** p, size_t bytes, bool host) {
    *p = nullptr;
    if (!host) return engine_malloc(p, std::max<size_t>(bytes, 16));
    if (alloc_refused()) return cudaErrorMemoryAllocation;
    void* hp = nullptr;
    cudaError_t e = cudaHostAlloc(&hp, std::max<size_t>(bytes, 16), cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) return e;
    void* dp = nullptr;
    e = cudaHostGetDevicePointer(&dp, hp, 0);
    if (e != cudaSuccess || dp != hp) {  // the kernels take the one pointer (unified addressing)
        cudaFreeHost(hp);
        return e != cudaSuccess ? e : cudaErrorInvalidValue;
    }
    *p = hp;
    return cudaSuccess;
}

bool gdfjk::is_host_memory(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void gdfjk::big_free(void* p) {
    if (!p) return;
    if (is_host_memory(p))
        cudaFreeHost(p);
    else
        cudaFree(p);
}

struct gdfjk_s {
    int device = 0;
    int nbf = 0, naux = 0, nT = 0, nbf_pad = 0, ntiles = 0;
    int flags = 0;
    std::vector<int> tI, tJ, map;
    cudaStream_t stream = nullptr;
    // J runs on its own stream, forked after D and joined before the build ends, so that its
    // FP64 / HBM-bound passes overlap the tensor-core K kernels on `stream`
    cudaStream_t stream_j = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool j_pending = false;
    int *d_tI = nullptr, *d_tJ = nullptr, *d_map = nullptr;
    int* d_err = nullptr;  // device-side error flag word
    double* B = nullptr;   // naux * ntiles * 4096
    bool B_ready = false;
    // workspaces
    int cap_nocc = -1;
    double *Cl = nullptr, *Cr = nullptr, *D = nullptr, *Dw = nullptr, *dq = nullptr, *Jt = nullptr;
    double *Xl = nullptr, *Xr = nullptr, *Kpart = nullptr, *Kt = nullptr;
    size_t Kpart_elems = 0;
    double *dJ = nullptr, *dK = nullptr, *dD = nullptr, *dCin = nullptr, *dCrin = nullptr;  // host-path staging
    size_t dCin_elems = 0;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    float t_j = 0, t_kt = 0, t_kc = 0;
    int cap_x = 0;               // nocc_pad the FP64 X buffers hold
    bool last_emulated = false;  // the last K went through the emulated-FP64 path
    int next_q = 0;              // next aux row expected by the block upload
    MixedState* mixed = nullptr;
    OzState* oz = nullptr;
    // backward workspaces
    double *gJp = nullptr, *gKp = nullptr, *Jg = nullptr, *Yb = nullptr, *Zpart = nullptr, *dCp = nullptr;
    double *gq = nullptr, *Dw2 = nullptr, *Jgt = nullptr, *hC = nullptr, *hgJ = nullptr, *hgK = nullptr, *hdC = nullptr,
           *hG = nullptr;
    int bw_cap_nocc = -1;
    std::string err;
};

namespace {

int set_err(gdfjk_t h, int code, const std::string& msg) {
    if (h)
        h->err = msg;
    else
        g_create_err = msg;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            return set_err(h, e_ == cudaErrorMemoryAllocation ? GDFJK_ERR_OOM : GDFJK_ERR_CUDA,      \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                      \
        }                                                                                            \
    } while (0)

template <class T>
int dalloc(gdfjk_t h, T** p, size_t n) {
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    if (n == 0) return GDFJK_OK;
    cudaError_t e = engine_malloc(reinterpret_cast<void**>(p), n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        char buf[160];
        snprintf(buf, sizeof buf, "device allocation of %.3f GB refused (%s)", n * sizeof(T) / 1e9,
                 cudaGetErrorString(e));
        return set_err(h, e == cudaErrorMemoryAllocation ? GDFJK_ERR_OOM : GDFJK_ERR_CUDA, buf);
    }
    return GDFJK_OK;
}

TileLayout layout_of(gdfjk_t h) { return TileLayout{h->nT, h->ntiles, h->d_tI, h->d_tJ, h->d_map}; }

// the FP64 tiles of B: HBM, or pinned Grace memory with GDFJK_B_HOST
int alloc_B(gdfjk_t h) {
    if (h->B) return GDFJK_OK;
    const size_t bytes = (size_t)h->naux * std::max(h->ntiles, 1) * TILE_ELEMS * sizeof(double);
    const bool host = (h->flags & GDFJK_B_HOST) != 0;
    cudaError_t e = big_alloc(reinterpret_cast<void**>(&h->B), bytes, host);
    if (e != cudaSuccess) {
        cudaGetLastError();
        h->B = nullptr;
        char buf[200];
        snprintf(buf, sizeof buf, "%s allocation of %.3f GB for B refused (%s)", host ? "pinned host" : "device",
                 bytes / 1e9, cudaGetErrorString(e));
        return set_err(h, e == cudaErrorMemoryAllocation ? GDFJK_ERR_OOM : GDFJK_ERR_CUDA, buf);
    }
    return GDFJK_OK;
}

// D/J work buffers and the padded C always; the FP64 X buffers and split-K partials only when
// `need_x` (the native FP64 K and the backward pass use them; the tensor-core forms do not).
int ensure_workspace(gdfjk_t h, int nocc_pad, bool nonsym, bool need_x) {
    int rc;
    size_t np2 = (size_t)h->nbf_pad * h->nbf_pad;
    // a group is (re)allocated whole unless every member exists, and a capacity is cleared
    // before its buffers are replaced, so that a refused allocation never leaves a buffer
    // missing behind a capacity that claims it
    if (!h->D || !h->Dw || !h->dq || !h->Jt || !h->Kt) {
        if ((rc = dalloc(h, &h->D, np2))) return rc;
        if ((rc = dalloc(h, &h->Dw, (size_t)std::max(h->ntiles, 1) * TILE_ELEMS))) return rc;
        if ((rc = dalloc(h, &h->dq, (size_t)std::max(h->naux, 1)))) return rc;
        if ((rc = dalloc(h, &h->Jt, (size_t)std::max(h->ntiles, 1) * TILE_ELEMS))) return rc;
        int nout_full = h->nT * h->nT;
        if ((rc = dalloc(h, &h->Kt, (size_t)nout_full * TILE_ELEMS))) return rc;
    }
    if (nocc_pad > h->cap_nocc) {
        h->cap_nocc = -1;
        if ((rc = dalloc(h, &h->Cl, (size_t)h->nbf_pad * std::max(nocc_pad, 1)))) return rc;
        if ((rc = dalloc(h, &h->Cr, (size_t)h->nbf_pad * std::max(nocc_pad, 1)))) return rc;
        h->cap_nocc = nocc_pad;
    }
    if (!need_x) return GDFJK_OK;
    if (nocc_pad > h->cap_x || (nonsym && !h->Xr && nocc_pad > 0)) {
        int cap = std::max(nocc_pad, h->cap_x);
        h->cap_x = 0;
        size_t xe = (size_t)h->nbf_pad * h->naux * cap;
        if ((rc = dalloc(h, &h->Xl, xe))) return rc;
        if (nonsym || h->Xr) {
            if ((rc = dalloc(h, &h->Xr, xe))) return rc;
        }
        h->cap_x = cap;
    }
    // split-K partials
    size_t kdim = (size_t)h->naux * std::max(nocc_pad, 1);
    int ns = k_contract_splits(h->nbf_pad, kdim, !nonsym);
    int nout = nonsym ? h->nT * h->nT : h->nT * (h->nT + 1) / 2;
    size_t need = (size_t)ns * nout * TILE_ELEMS;
    if (need > h->Kpart_elems) {
        h->Kpart_elems = 0;
        if ((rc = dalloc(h, &h->Kpart, need))) return rc;
        h->Kpart_elems = need;
    }
    return GDFJK_OK;
}

}  // namespace

namespace {

// Enqueue one build on the handle's stream; all pointers are device pointers.
// J (when asked) goes to h->stream_j after D, so that its two HBM-bound passes over B fill the
// SMs the tensor-core K kernels leave idle (the tail waves of the half-transform, the
// contraction, the reductions).  The native FP64 K, FP64-pipe work like J, runs after J on the
// one stream.  J joins h->stream at the end (join = false leaves the join to the caller: join_j).
constexpr double J_FORK_MIN_BYTES = 8e9;  // B of at least this size: J on the second stream

void join_j(gdfjk_t h) {
    if (h->j_pending) {
        cudaStreamWaitEvent(h->stream, h->ev_join, 0);
        h->j_pending = false;
    }
}

int enqueue_build(gdfjk_t h, const double* C_left, const double* C_right, int nocc, int ldc, int mode, double* D_out,
                  double* J, double* K, bool join = true, bool reuse_C = false) {
    const bool do_J = mode & GDFJK_DO_J;
    const bool do_K = mode & GDFJK_DO_K;
    const bool nonsym = C_right != nullptr;
    const int nocc_pad = round_up(std::max(nocc, 0), 32);
    if (mode & GDFJK_DO_K) h->last_emulated = false;
    const bool native_k = do_K && nocc > 0 && !(mode & GDFJK_MIXED) && !(mode & GDFJK_EMULATED);
    int rc = ensure_workspace(h, nocc_pad, nonsym, native_k);
    if (rc == GDFJK_ERR_OOM && native_k) {  // the FP64 X workspace: give both tensor-core forms' copies back, retry
        CK(cudaStreamSynchronize(h->stream));
        mixed_release(h->mixed);
        oz_release(h->oz);
        rc = ensure_workspace(h, nocc_pad, nonsym, native_k);
    }
    if (rc) return rc;
    cudaStream_t s = h->stream;
    TileLayout L = layout_of(h);
    CK(cudaEventRecord(h->ev[0], s));
    // C padded to nbf_pad x nocc_pad (reuse_C: the previous build on this stream padded the
    // same C into h->Cl, and nothing has written it since)
    if (nocc_pad > 0 && !reuse_C) {
        launch_pad_C(C_left, h->nbf, nocc, ldc, h->nbf_pad, nocc_pad, h->Cl, s);
        if (nonsym) launch_pad_C(C_right, h->nbf, nocc, ldc, h->nbf_pad, nocc_pad, h->Cr, s);
    }
    // D = C_left C_right^T (FP64, ~1 ms at nbf 1856): only J and the caller read it, no K path
    // does.  It stays on K's stream ahead of the fork: on J's lowest-priority stream the K
    // kernels starve it and J starts late (the mixed C2 build went from 42.8 to 49.0 ms)
    if (do_J || D_out) launch_density(h->Cl, nonsym ? h->Cr : h->Cl, h->nbf_pad, nocc_pad, h->D, s);
    if (D_out) launch_copy_out(h->D, h->nbf, h->nbf_pad, D_out, s);
    // J on the second stream only beside a tensor-core K (or alone, when the caller joins
    // later) and only on a large B.  Measured on one GB300: at nbf 1856 / naux 4448 (61 GB of
    // B) the emulated build went from 224 to 215 ms; at nbf 384 / naux 1856 (1.3 GB, J well
    // under a millisecond) it went from 4.7 to 5.0 ms
    const bool tc_k = !do_K || (mode & (GDFJK_MIXED | GDFJK_EMULATED));
    const bool fork = do_J && tc_k && (double)h->naux * h->ntiles * 4096 * sizeof(double) >= J_FORK_MIN_BYTES;
    cudaStream_t sj = fork ? h->stream_j : s;
    if (fork) {
        CK(cudaEventRecord(h->ev_fork, s));
        CK(cudaStreamWaitEvent(sj, h->ev_fork, 0));
    }
    if (do_J) {
        launch_weighted_density_tiles(h->D, h->nbf_pad, L, h->Dw, sj);
        launch_j_pass1(h->B, h->Dw, h->naux, L, h->dq, sj);
        launch_j_pass2(h->B, h->dq, h->naux, L, h->Jt, sj);
        launch_unpack_tiles(h->Jt, L, h->nbf, h->nbf_pad, J, h->nbf, true, sj);
        CK(cudaEventRecord(h->ev[1], sj));
        if (fork) {
            CK(cudaEventRecord(h->ev_join, sj));
            h->j_pending = true;
        }
    } else {
        CK(cudaEventRecord(h->ev[1], s));
    }
    CK(cudaEventRecord(h->ev[2], s));
    if (do_K) {
        if (nocc == 0) {
            CK(cudaMemsetAsync(K, 0, sizeof(double) * (size_t)h->nbf * h->nbf, s));
            CK(cudaEventRecord(h->ev[3], s));
        } else if (mode & GDFJK_MIXED) {
            if (nonsym) {
                join_j(h);
                return set_err(h, GDFJK_ERR_ARG, "mixed-precision K needs an lr-symmetric density");
            }
            rc = mixed_build_K(h->mixed, h->B, L, h->map.data(), h->nbf, h->nbf_pad, h->naux, h->Cl, nocc, nocc_pad, mode, K,
                               h->ev[3], s, h->err);
            if (rc == GDFJK_ERR_OOM) {  // give the emulated form's caches back and retry once
                CK(cudaStreamSynchronize(s));
                oz_release(h->oz);
                rc = mixed_build_K(h->mixed, h->B, L, h->map.data(), h->nbf, h->nbf_pad, h->naux, h->Cl, nocc, nocc_pad, mode, K,
                                   h->ev[3], s, h->err);
            }
            if (rc) {
                join_j(h);
                return rc;
            }
        } else if (mode & GDFJK_EMULATED) {
            h->last_emulated = true;
            const double* Cr = nonsym ? h->Cr : nullptr;
            rc = oz_build_K(h->oz, h->B, L, h->map.data(), h->nbf, h->naux, h->Cl, Cr, nocc, nocc_pad, K, h->ev[3], s,
                            h->err);
            if (rc == GDFJK_ERR_OOM) {  // give the mixed form's split copy of B back and retry once
                CK(cudaStreamSynchronize(s));
                mixed_release(h->mixed);
                rc = oz_build_K(h->oz, h->B, L, h->map.data(), h->nbf, h->naux, h->Cl, Cr, nocc, nocc_pad, K, h->ev[3], s,
                                h->err);
            }
            if (rc) {
                join_j(h);
                return rc;
            }
        } else {
            launch_k_transform_fp64(h->B, h->Cl, h->naux, h->nbf_pad, nocc_pad, L, h->Xl, s);
            if (nonsym) launch_k_transform_fp64(h->B, h->Cr, h->naux, h->nbf_pad, nocc_pad, L, h->Xr, s);
            CK(cudaEventRecord(h->ev[3], s));
            size_t kdim = (size_t)h->naux * nocc_pad;
            int ns = k_contract_splits(h->nbf_pad, kdim, !nonsym);
            launch_k_contract_fp64(h->Xl, nonsym ? h->Xr : h->Xl, h->nbf_pad, kdim, !nonsym, L, h->Kpart, ns, h->Kt, s);
            if (nonsym)
                launch_unpack_tiles(h->Kt, L, h->nbf, h->nbf_pad, K, h->nbf, false, s);
            else
                launch_unpack_lower_full(h->Kt, h->nT, h->nbf, K, h->nbf, s);
        }
    } else {
        CK(cudaEventRecord(h->ev[3], s));
    }
    if (join) join_j(h);
    CK(cudaEventRecord(h->ev[4], s));
    CK(cudaGetLastError());
    return GDFJK_OK;
}

int wait_stream(gdfjk_t h, double timeout_s) {
    auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaStreamQuery(h->stream);
        if (e == cudaSuccess) return GDFJK_OK;
        if (e != cudaErrorNotReady) return set_err(h, GDFJK_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s > 0 && el > timeout_s) {
            char buf[128];
            snprintf(buf, sizeof buf, "stream did not finish within %.1f s", timeout_s);
            return set_err(h, GDFJK_ERR_TIMEOUT, buf);
        }
        std::this_thread::sleep_for(std::chrono::microseconds(el < 0.01 ? 20 : 500));
    }
}

int check_device_flag(gdfjk_t h) {
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    flag |= mixed_error_flag(h->mixed, h->stream);
    flag |= oz_error_flag(h->oz, h->stream);
    if (flag) {
        CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
        if (flag & 4) return set_err(h, GDFJK_ERR_NUMERIC, "non-finite values in J or K");
        return set_err(h, GDFJK_ERR_DEVICE, "a kernel reported an internal error (flag " + std::to_string(flag) + ")");
    }
    return GDFJK_OK;
}

double env_timeout() {
    const char* s = getenv("GDFJK_TIMEOUT_S");
    return s ? atof(s) : 600.0;
}

}  // namespace

extern "C" {

const char* gdfjk_last_error(gdfjk_t h) { return h ? h->err.c_str() : g_create_err.c_str(); }

int gdfjk_query_memory(int nbf, int naux, int max_nocc, int flags, size_t* bytes) {
    if (nbf <= 0 || naux <= 0 || max_nocc < 0 || !bytes) return set_err(nullptr, GDFJK_ERR_ARG, "query_memory: bad sizes");
    int nT = (nbf + TILE - 1) / TILE;
    size_t nbf_pad = (size_t)nT * TILE;
    size_t ntiles = (size_t)nT * (nT + 1) / 2;  // upper bound (no screening)
    size_t nocc_pad = (size_t)round_up(max_nocc, 32);
    size_t b = (flags & GDFJK_B_HOST) ? 0 : (size_t)naux * ntiles * TILE_ELEMS * 8;  // B (HBM)
    b += nbf_pad * nbf_pad * 8 + 2 * ntiles * TILE_ELEMS * 8;    // D, Dw, Jt
    b += (size_t)nT * nT * TILE_ELEMS * 8 + naux * 8;            // Kt, dq
    b += nbf_pad * naux * nocc_pad * 8;                          // X
    b += 2 * nbf_pad * nocc_pad * 8;                             // C
    int ns = k_contract_splits((int)nbf_pad, (size_t)naux * std::max<size_t>(nocc_pad, 1), true);
    b += (size_t)ns * ntiles * TILE_ELEMS * 8;                   // split-K partials
    if (flags & GDFJK_MIXED) b += mixed_query_memory(nbf, naux, max_nocc);
    if (flags & GDFJK_EMULATED) b += oz_query_memory(nbf, naux, max_nocc);
    *bytes = b;
    return GDFJK_OK;
}

int gdfjk_create(int device, int nbf, int naux, const unsigned char* pair_mask, int flags, gdfjk_t* out) {
    if (!out) return set_err(nullptr, GDFJK_ERR_ARG, "create: out is NULL");
    *out = nullptr;
    if (nbf <= 0 || naux <= 0) return set_err(nullptr, GDFJK_ERR_ARG, "create: nbf and naux must be positive");
    if (naux > 65535) return set_err(nullptr, GDFJK_ERR_ARG, "create: naux above 65535 is not supported");
    gdfjk_t h = new gdfjk_s();
    h->device = device;
    h->nbf = nbf;
    h->naux = naux;
    h->flags = flags;
    h->nT = (nbf + TILE - 1) / TILE;
    h->nbf_pad = h->nT * TILE;
    // tile list: (I, J), I >= J, holding at least one significant pair
    h->map.assign((size_t)h->nT * h->nT, -1);
    for (int I = 0; I < h->nT; ++I)
        for (int J = 0; J <= I; ++J) {
            bool any = false;
            if (!pair_mask) {
                any = true;
            } else {
                for (int r = 0; r < TILE && !any; ++r)
                    for (int c = 0; c < TILE && !any; ++c) {
                        int m = I * TILE + r, n = J * TILE + c;
                        if (m < nbf && n < nbf && pair_mask[(size_t)m * nbf + n]) any = true;
                    }
            }
            if (any) {
                h->map[(size_t)I * h->nT + J] = (int)h->tI.size();
                h->tI.push_back(I);
                h->tJ.push_back(J);
            }
        }
    h->ntiles = (int)h->tI.size();
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        std::string m = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        delete h;
        return set_err(nullptr, GDFJK_ERR_CUDA, m);
    }
    int rc = GDFJK_OK;
    auto fail = [&](int code) {
        g_create_err = h->err;
        gdfjk_destroy(h);
        return code;
    };
    // K's stream at the highest priority, J's at the lowest: when an SM frees resources the
    // block scheduler places K's persistent CTAs first and J's small blocks in what is left
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&h->stream_j, cudaStreamNonBlocking, prio_least) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        h->err = "cudaStreamCreate failed";
        return fail(GDFJK_ERR_CUDA);
    }
    for (auto& ev : h->ev)
        if (cudaEventCreate(&ev) != cudaSuccess) {
            h->err = "cudaEventCreate failed";
            return fail(GDFJK_ERR_CUDA);
        }
    if ((rc = dalloc(h, &h->d_tI, std::max<size_t>(h->ntiles, 1)))) return fail(rc);
    if ((rc = dalloc(h, &h->d_tJ, std::max<size_t>(h->ntiles, 1)))) return fail(rc);
    if ((rc = dalloc(h, &h->d_map, h->map.size()))) return fail(rc);
    if ((rc = dalloc(h, &h->d_err, 1))) return fail(rc);
    if (h->ntiles) {
        cudaMemcpy(h->d_tI, h->tI.data(), sizeof(int) * h->ntiles, cudaMemcpyHostToDevice);
        cudaMemcpy(h->d_tJ, h->tJ.data(), sizeof(int) * h->ntiles, cudaMemcpyHostToDevice);
    }
    cudaMemcpy(h->d_map, h->map.data(), sizeof(int) * h->map.size(), cudaMemcpyHostToDevice);
    cudaMemset(h->d_err, 0, sizeof(int));
    h->mixed = mixed_create();
    h->oz = oz_create();

    if (cudaGetLastError() != cudaSuccess) {
        h->err = "create: CUDA error while initialising";
        return fail(GDFJK_ERR_CUDA);
    }
    *out = h;
    return GDFJK_OK;
}

int gdfjk_destroy(gdfjk_t h) {
    if (!h) return GDFJK_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->stream_j) cudaStreamSynchronize(h->stream_j);
    big_free(h->B);
    double* bufs[] = {h->Cl,  h->Cr,  h->D,     h->Dw,  h->dq,  h->Jt,  h->Xl, h->Xr,  h->Kpart,
                      h->Kt,  h->dJ,  h->dK,  h->dD,    h->dCin, h->dCrin, h->gJp, h->gKp, h->Jg, h->Yb,
                      h->Zpart, h->dCp, h->gq, h->Dw2, h->Jgt, h->hC,  h->hgJ, h->hgK, h->hdC, h->hG};
    for (double* p : bufs)
        if (p) cudaFree(p);
    if (h->d_tI) cudaFree(h->d_tI);
    if (h->d_tJ) cudaFree(h->d_tJ);
    if (h->d_map) cudaFree(h->d_map);
    if (h->d_err) cudaFree(h->d_err);
    mixed_destroy(h->mixed);
    oz_destroy(h->oz);
    for (auto& ev : h->ev)
        if (ev) cudaEventDestroy(ev);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->stream_j) cudaStreamDestroy(h->stream_j);
    delete h;
    return GDFJK_OK;
}

void* gdfjk_stream(gdfjk_t h) { return h ? (void*)h->stream : nullptr; }

// Rows [q0, q0 + nq) of the packed triangle, device pointer, into the stored tiles.
static int upload_rows_device(gdfjk_t h, const double* Bq, int q0, int nq) {
    int rc;
    if (q0 == 0) {
        if (!h->B) {
            if ((rc = alloc_B(h))) return rc;
        }
        h->B_ready = false;
        mixed_invalidate(h->mixed);
        oz_invalidate(h->oz);
        h->next_q = 0;
    }
    if (q0 != h->next_q) return set_err(h, GDFJK_ERR_STATE, "upload_B_block: blocks must follow each other from q0 = 0");
    TileLayout L = layout_of(h);
    launch_relayout_qtri(Bq, q0, nq, h->nbf, L, h->B, h->stream);
    CK(cudaGetLastError());
    if ((rc = wait_stream(h, env_timeout()))) return rc;
    h->next_q = q0 + nq;
    if (h->next_q == h->naux) h->B_ready = true;
    return GDFJK_OK;
}

int gdfjk_upload_B_device_block(gdfjk_t h, const double* Bq, int q0, int nq) {
    if (!h || !Bq) return set_err(h, GDFJK_ERR_ARG, "upload_B_device_block: null argument");
    if (q0 < 0 || nq <= 0 || q0 + nq > h->naux) return set_err(h, GDFJK_ERR_ARG, "upload_B_device_block: bad q0 / nq");
    CK(cudaSetDevice(h->device));
    return upload_rows_device(h, Bq, q0, nq);
}

int gdfjk_upload_B_block(gdfjk_t h, const double* Bq, int q0, int nq) {
    if (!h || !Bq) return set_err(h, GDFJK_ERR_ARG, "upload_B_block: null argument");
    if (q0 < 0 || nq <= 0 || q0 + nq > h->naux) return set_err(h, GDFJK_ERR_ARG, "upload_B_block: bad q0 / nq");
    CK(cudaSetDevice(h->device));
    const size_t npair = (size_t)h->nbf * (h->nbf + 1) / 2;
    // staged through the host-path buffer in sub-blocks of at most 512 MB
    const int sub = (int)std::max<size_t>(1, std::min<size_t>((size_t)nq, (size_t)(512u << 20) / (npair * 8)));
    double* stage = nullptr;
    if (engine_malloc((void**)&stage, (size_t)sub * npair * 8) != cudaSuccess) {
        cudaGetLastError();
        return set_err(h, GDFJK_ERR_OOM, "upload_B_block: staging buffer refused");
    }
    int rc = GDFJK_OK;
    for (int k = 0; k < nq && rc == GDFJK_OK; k += sub) {
        const int n = std::min(sub, nq - k);
        if (cudaMemcpyAsync(stage, Bq + (size_t)k * npair, (size_t)n * npair * 8, cudaMemcpyHostToDevice, h->stream) !=
            cudaSuccess) {
            rc = set_err(h, GDFJK_ERR_CUDA, "upload_B_block: host-to-device copy failed");
            break;
        }
        rc = upload_rows_device(h, stage, q0 + k, n);
    }
    cudaStreamSynchronize(h->stream);
    cudaFree(stage);
    return rc;
}

int gdfjk_upload_B_device(gdfjk_t h, const double* Bq) {
    if (!h || !Bq) return set_err(h, GDFJK_ERR_ARG, "upload_B_device: null argument");
    CK(cudaSetDevice(h->device));
    int rc;
    if (!h->B) {
        if ((rc = alloc_B(h))) return rc;
    }
    TileLayout L = layout_of(h);
    const int chunk = 4096;
    size_t npair = (size_t)h->nbf * (h->nbf + 1) / 2;
    for (int q0 = 0; q0 < h->naux; q0 += chunk) {
        int nq = std::min(chunk, h->naux - q0);
        launch_relayout_qtri(Bq + (size_t)q0 * npair, q0, nq, h->nbf, L, h->B, h->stream);
    }
    CK(cudaGetLastError());
    if ((rc = wait_stream(h, env_timeout()))) return rc;
    mixed_invalidate(h->mixed);
    oz_invalidate(h->oz);
    h->B_ready = true;
    return GDFJK_OK;
}

int gdfjk_metric_contract_device(gdfjk_t h, const double* metric, const double* Pmn, int ncols, int64_t ldp, double* B,
                                 int64_t ldb, int accumulate) {
    if (!h || !metric || !Pmn || !B) return set_err(h, GDFJK_ERR_ARG, "metric_contract_device: null argument");
    if (ncols < 0 || ldp < ncols || ldb < ncols)
        return set_err(h, GDFJK_ERR_ARG, "metric_contract_device: invalid column count or leading dimension");
    CK(cudaSetDevice(h->device));
    if (!h->oz) h->oz = oz_create();
    int rc = oz_gemm(h->oz, metric, (size_t)h->naux, Pmn, (size_t)ldp, B, (size_t)ldb, h->naux, ncols, h->naux,
                     accumulate, h->stream, h->err);
    if (rc) return set_err(h, rc, "metric_contract_device: " + h->err);
    return check_device_flag(h);
}

int gdfjk_gemm_device(gdfjk_t h, int transb, int M, int N, int K, const double* A, int64_t lda, const double* B,
                      int64_t ldb, double* C, int64_t ldc, int accumulate) {
    if (!h || !A || !B || !C) return set_err(h, GDFJK_ERR_ARG, "gemm_device: null argument");
    if (M < 0 || N < 0 || K < 1 || lda < K || ldb < (transb ? K : N) || ldc < N)
        return set_err(h, GDFJK_ERR_ARG, "gemm_device: invalid sizes or leading dimensions");
    CK(cudaSetDevice(h->device));
    if (!h->oz) h->oz = oz_create();
    int rc = oz_gemm(h->oz, A, (size_t)lda, B, (size_t)ldb, C, (size_t)ldc, M, N, K, accumulate, h->stream, h->err,
                     transb ? 1 : 0);
    if (rc) return set_err(h, rc, "gemm_device: " + h->err);
    return check_device_flag(h);
}

int gdfjk_upload_B(gdfjk_t h, const double* B, int layout, const int64_t* big_skips, const int64_t* small_skips,
                   const int64_t* fun_index) {
    if (!h || !B) return set_err(h, GDFJK_ERR_ARG, "upload_B: null argument");
    if (layout != GDFJK_LAYOUT_PQQ && layout != GDFJK_LAYOUT_QTRI)
        return set_err(h, GDFJK_ERR_ARG, "upload_B: unknown layout");
    if (layout == GDFJK_LAYOUT_PQQ && (!big_skips || !small_skips || !fun_index))
        return set_err(h, GDFJK_ERR_ARG, "upload_B: the pQq layout needs big_skips, small_skips and fun_index");
    CK(cudaSetDevice(h->device));
    int rc;
    if (!h->B) {
        if ((rc = alloc_B(h))) return rc;
    }
    const size_t nbf = h->nbf;
    const size_t npair = nbf * (nbf + 1) / 2;
    // chunk of Q rows staged as packed triangles: about 256 MB per buffer
    int chunk = (int)std::max<size_t>(1, std::min<size_t>(h->naux, (256ull << 20) / (npair * 8)));
    double* host_stage[2] = {nullptr, nullptr};
    double* dev_stage[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    auto cleanup = [&]() {
        for (int k = 0; k < 2; ++k) {
            if (host_stage[k]) cudaFreeHost(host_stage[k]);
            if (dev_stage[k]) cudaFree(dev_stage[k]);
            if (done[k]) cudaEventDestroy(done[k]);
        }
    };
    for (int k = 0; k < 2; ++k) {
        if (alloc_refused() || cudaMallocHost(&host_stage[k], (size_t)chunk * npair * 8) != cudaSuccess ||
            engine_malloc((void**)&dev_stage[k], (size_t)chunk * npair * 8) != cudaSuccess ||
            cudaEventCreate(&done[k]) != cudaSuccess) {
            cudaGetLastError();
            cleanup();
            return set_err(h, GDFJK_ERR_OOM, "upload_B: staging allocation refused");
        }
    }
    TileLayout L = layout_of(h);
    unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    int buf = 0;
    for (int q0 = 0; q0 < h->naux; q0 += chunk, buf ^= 1) {
        int nq = std::min(chunk, h->naux - q0);
        cudaEventSynchronize(done[buf]);  // staging buffer free again
        double* st = host_stage[buf];
        // gather this chunk into packed triangles on the host
        auto work = [&](unsigned tid) {
            for (size_t m = tid; m < nbf; m += nth) {
                for (int qq = 0; qq < nq; ++qq) {
                    double* dst = st + (size_t)qq * npair + m * (m + 1) / 2;
                    size_t Q = (size_t)(q0 + qq);
                    if (layout == GDFJK_LAYOUT_QTRI) {
                        std::memcpy(dst, B + Q * npair + m * (m + 1) / 2, (m + 1) * sizeof(double));
                    } else {
                        // pQq row m: B[big_skips[m] + Q*small_skips[m] + fun_index[m][n]-1]
                        const double* row = B + big_skips[m] + Q * small_skips[m];
                        const int64_t* fi = fun_index + m * nbf;
                        for (size_t n = 0; n <= m; ++n) dst[n] = fi[n] ? row[fi[n] - 1] : 0.0;
                    }
                }
            }
        };
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nth; ++t) pool.emplace_back(work, t);
        work(0);
        for (auto& th : pool) th.join();
        if (cudaMemcpyAsync(dev_stage[buf], st, (size_t)nq * npair * 8, cudaMemcpyHostToDevice, h->stream) !=
            cudaSuccess) {
            cleanup();
            return set_err(h, GDFJK_ERR_CUDA, "upload_B: host-to-device copy failed");
        }
        launch_relayout_qtri(dev_stage[buf], q0, nq, h->nbf, L, h->B, h->stream);
        cudaEventRecord(done[buf], h->stream);
    }
    cudaError_t e = cudaGetLastError();
    rc = wait_stream(h, env_timeout());
    cleanup();
    if (e != cudaSuccess) return set_err(h, GDFJK_ERR_CUDA, std::string("upload_B: ") + cudaGetErrorString(e));
    if (rc) return rc;
    mixed_invalidate(h->mixed);
    oz_invalidate(h->oz);
    h->B_ready = true;
    return GDFJK_OK;
}

int gdfjk_compute_device(gdfjk_t h, const double* C_left, const double* C_right, int nocc, int ldc, int mode,
                         double* D_out, double* J, double* K) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "compute: null handle");
    if (!h->B_ready) return set_err(h, GDFJK_ERR_STATE, "compute: B has not been uploaded (call gdfjk_upload_B first)");
    if (nocc < 0 || (nocc > 0 && (!C_left || ldc < nocc))) return set_err(h, GDFJK_ERR_ARG, "compute: bad C / nocc / ldc");
    if ((mode & GDFJK_DO_J) && !J) return set_err(h, GDFJK_ERR_ARG, "compute: J output is NULL");
    if ((mode & GDFJK_DO_K) && !K) return set_err(h, GDFJK_ERR_ARG, "compute: K output is NULL");
    CK(cudaSetDevice(h->device));
    return enqueue_build(h, C_left, C_right, nocc, ldc, mode, D_out, J, K);
}

int gdfjk_compute(gdfjk_t h, const double* C_left, const double* C_right, int nocc, int ldc, int mode, double* D_out,
                  double* J, double* K) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "compute: null handle");
    if (!h->B_ready) return set_err(h, GDFJK_ERR_STATE, "compute: B has not been uploaded (call gdfjk_upload_B first)");
    if (nocc < 0 || (nocc > 0 && (!C_left || ldc < nocc))) return set_err(h, GDFJK_ERR_ARG, "compute: bad C / nocc / ldc");
    if ((mode & GDFJK_DO_J) && !J) return set_err(h, GDFJK_ERR_ARG, "compute: J output is NULL");
    if ((mode & GDFJK_DO_K) && !K) return set_err(h, GDFJK_ERR_ARG, "compute: K output is NULL");
    CK(cudaSetDevice(h->device));
    int rc;
    size_t n2 = (size_t)h->nbf * h->nbf;
    size_t cin = (size_t)h->nbf * std::max(ldc, 1);
    if (!h->dJ || !h->dK || !h->dD) {
        if ((rc = dalloc(h, &h->dJ, n2))) return rc;
        if ((rc = dalloc(h, &h->dK, n2))) return rc;
        if ((rc = dalloc(h, &h->dD, n2))) return rc;
    }
    if (cin > h->dCin_elems) {
        h->dCin_elems = 0;
        if ((rc = dalloc(h, &h->dCin, cin))) return rc;
        if ((rc = dalloc(h, &h->dCrin, cin))) return rc;
        h->dCin_elems = cin;
    }
    cudaStream_t s = h->stream;
    if (nocc > 0) {
        CK(cudaMemcpyAsync(h->dCin, C_left, cin * 8, cudaMemcpyHostToDevice, s));
        if (C_right) CK(cudaMemcpyAsync(h->dCrin, C_right, cin * 8, cudaMemcpyHostToDevice, s));
    }
    rc = enqueue_build(h, nocc > 0 ? h->dCin : nullptr, C_right ? h->dCrin : nullptr, nocc, std::max(ldc, 1), mode,
                       D_out ? h->dD : nullptr, h->dJ, h->dK);
    if (rc) return rc;
    if (mode & GDFJK_DO_J) launch_finite_check(h->dJ, n2, h->d_err, s);
    if (mode & GDFJK_DO_K) launch_finite_check(h->dK, n2, h->d_err, s);
    if (mode & GDFJK_DO_J) CK(cudaMemcpyAsync(J, h->dJ, n2 * 8, cudaMemcpyDeviceToHost, s));
    if (mode & GDFJK_DO_K) CK(cudaMemcpyAsync(K, h->dK, n2 * 8, cudaMemcpyDeviceToHost, s));
    if (D_out) CK(cudaMemcpyAsync(D_out, h->dD, n2 * 8, cudaMemcpyDeviceToHost, s));
    if ((rc = wait_stream(h, env_timeout()))) return rc;
    return check_device_flag(h);
}

int gdfjk_compute_wK(gdfjk_t hl, gdfjk_t hr, const double* C_left, const double* C_right, int nocc, int ldc, int mode,
                     double* wK) {
    if (!hl || !hr || !wK) return set_err(hl, GDFJK_ERR_ARG, "compute_wK: null handle or output");
    if (hl->nbf != hr->nbf || hl->naux != hr->naux || hl->map != hr->map || hl->device != hr->device)
        return set_err(hl, GDFJK_ERR_ARG, "compute_wK: the two handles must share nbf, naux, the pair mask and the device");
    if (!hl->B_ready || !hr->B_ready) return set_err(hl, GDFJK_ERR_STATE, "compute_wK: upload both tensors first");
    if (nocc < 0 || (nocc > 0 && (!C_left || ldc < nocc))) return set_err(hl, GDFJK_ERR_ARG, "compute_wK: bad C / nocc / ldc");
    gdfjk_t h = hl;  // workspaces and stream of the left handle
    CK(cudaSetDevice(h->device));
    int rc;
    const size_t n2 = (size_t)h->nbf * h->nbf;
    const size_t cin = (size_t)h->nbf * std::max(ldc, 1);
    if (!h->dJ || !h->dK || !h->dD) {
        if ((rc = dalloc(h, &h->dJ, n2))) return rc;
        if ((rc = dalloc(h, &h->dK, n2))) return rc;
        if ((rc = dalloc(h, &h->dD, n2))) return rc;
    }
    if (cin > h->dCin_elems) {
        h->dCin_elems = 0;
        if ((rc = dalloc(h, &h->dCin, cin))) return rc;
        if ((rc = dalloc(h, &h->dCrin, cin))) return rc;
        h->dCin_elems = cin;
    }
    cudaStream_t s = h->stream;
    if (nocc == 0) {
        std::fill(wK, wK + n2, 0.0);
        return GDFJK_OK;
    }
    const bool lr = C_right == nullptr;
    CK(cudaMemcpyAsync(h->dCin, C_left, cin * 8, cudaMemcpyHostToDevice, s));
    if (!lr) CK(cudaMemcpyAsync(h->dCrin, C_right, cin * 8, cudaMemcpyHostToDevice, s));
    const int nocc_pad = round_up(nocc, 32);
    const bool emulated = (mode & GDFJK_EMULATED) != 0;
    if ((rc = ensure_workspace(h, nocc_pad, true, !emulated))) return rc;
    launch_pad_C(h->dCin, h->nbf, nocc, ldc, h->nbf_pad, nocc_pad, h->Cl, s);
    launch_pad_C(lr ? h->dCin : h->dCrin, h->nbf, nocc, ldc, h->nbf_pad, nocc_pad, h->Cr, s);
    TileLayout L = layout_of(h), Lr = layout_of(hr);
    if (emulated) {
        h->last_emulated = true;
        rc = oz_build_K(h->oz, h->B, L, h->map.data(), h->nbf, h->naux, h->Cl, h->Cr, nocc, nocc_pad, h->dK, nullptr, s,
                        h->err, hr->oz, hr->B, &Lr);
        if (rc) return set_err(h, rc, h->err);
    } else {
        h->last_emulated = false;
        launch_k_transform_fp64(h->B, h->Cl, h->naux, h->nbf_pad, nocc_pad, L, h->Xl, s);
        launch_k_transform_fp64(hr->B, h->Cr, h->naux, h->nbf_pad, nocc_pad, Lr, h->Xr, s);
        const size_t kdim = (size_t)h->naux * nocc_pad;
        const int ns = k_contract_splits(h->nbf_pad, kdim, false);
        launch_k_contract_fp64(h->Xl, h->Xr, h->nbf_pad, kdim, false, L, h->Kpart, ns, h->Kt, s);
        launch_unpack_tiles(h->Kt, L, h->nbf, h->nbf_pad, h->dK, h->nbf, false, s);
    }
    launch_finite_check(h->dK, n2, h->d_err, s);
    CK(cudaMemcpyAsync(wK, h->dK, n2 * 8, cudaMemcpyDeviceToHost, s));
    if ((rc = wait_stream(h, env_timeout()))) return rc;
    if ((rc = check_device_flag(h))) return rc;
    if (lr) {  // MemDFJK::compute_JK hermitivitizes wK for lr-symmetric densities (MemDFJK.cc:103-108)
        const size_t n = (size_t)h->nbf;
        for (size_t m = 0; m < n; ++m)
            for (size_t k = 0; k < m; ++k) {
                const double v = 0.5 * (wK[m * n + k] + wK[k * n + m]);
                wK[m * n + k] = v;
                wK[k * n + m] = v;
            }
    }
    return GDFJK_OK;
}

}  // extern "C"

namespace {

int check_incremental_args(gdfjk_t h, const double* C, int nocc, int ldc, const double* U, int nu, int npos, int ldu,
                           int mode, const double* J, const double* K) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "compute_incremental: null handle");
    if (!h->B_ready) return set_err(h, GDFJK_ERR_STATE, "compute_incremental: B has not been uploaded");
    if (nocc < 0 || (nocc > 0 && (!C || ldc < nocc))) return set_err(h, GDFJK_ERR_ARG, "compute_incremental: bad C / nocc / ldc");
    if (nu < 0 || npos < 0 || npos > nu || (nu > 0 && (!U || ldu < nu)))
        return set_err(h, GDFJK_ERR_ARG, "compute_incremental: bad U / nu / npos / ldu");
    if ((mode & GDFJK_DO_J) && !J) return set_err(h, GDFJK_ERR_ARG, "compute_incremental: J output is NULL");
    if ((mode & GDFJK_DO_K) && !K) return set_err(h, GDFJK_ERR_ARG, "compute_incremental: K output is NULL");
    return GDFJK_OK;
}

// The incremental build on the handle's stream, all pointers on the device: J (FP64) from C;
// K either a full FP64 anchor from C (kept as the base) or the base plus the split-BF16
// increment of the factor U.
int enqueue_incremental(gdfjk_t h, const double* C, int nocc, int ldc, const double* U, int nu, int npos, int ldu,
                        int mode, double* J, double* K) {
    int rc;
    const size_t n2 = (size_t)h->nbf * h->nbf;
    cudaStream_t s = h->stream;
    if (mode & GDFJK_DO_J) {
        // J on its own stream, joined after K below so that the two overlap
        rc = enqueue_build(h, nocc > 0 ? C : nullptr, nullptr, nocc, std::max(ldc, 1), GDFJK_DO_J, nullptr, J, nullptr,
                           false);
        if (rc) {
            join_j(h);
            return rc;
        }
    }
    if ((mode & GDFJK_DO_K) && !(mode & GDFJK_MIXED)) {
        // FP64 anchor: a full FP64 K from C that becomes the base of later increments (its C
        // is the one the J build above padded: not padded again while J may still read it)
        rc = enqueue_build(h, nocc > 0 ? C : nullptr, nullptr, nocc, std::max(ldc, 1), GDFJK_DO_K | (mode & GDFJK_EMULATED),
                           nullptr, nullptr, K, true, (mode & GDFJK_DO_J) != 0);
        if (rc) return rc;
        rc = mixed_set_base(h->mixed, K, h->nbf, s, h->err);
        if (rc) return rc;
        launch_finite_check(K, n2, h->d_err, s);
    } else if (mode & GDFJK_DO_K) {
        CK(cudaEventRecord(h->ev[2], s));
        auto factor = [&]() {
            return mixed_k_factor(h->mixed, h->B, layout_of(h), h->map.data(), h->nbf, h->naux, U, std::max(ldu, 1), npos,
                                  nu - npos, (mode & GDFJK_RESET) ? 0 : 1, K, h->ev[3], s, h->err);
        };
        rc = factor();
        if (rc == GDFJK_ERR_OOM) {  // give the emulated form's caches back and retry once
            CK(cudaStreamSynchronize(s));
            oz_release(h->oz);
            rc = factor();
        }
        if (rc) return rc;
        CK(cudaEventRecord(h->ev[4], s));
        launch_finite_check(K, n2, h->d_err, s);
    }
    if (mode & GDFJK_DO_J) {
        join_j(h);
        launch_finite_check(J, n2, h->d_err, s);
    }
    CK(cudaGetLastError());
    return GDFJK_OK;
}

}  // namespace

extern "C" {

int gdfjk_compute_incremental(gdfjk_t h, const double* C, int nocc, int ldc, const double* U, int nu, int npos, int ldu,
                              int mode, double* J, double* K) {
    int rc = check_incremental_args(h, C, nocc, ldc, U, nu, npos, ldu, mode, J, K);
    if (rc) return rc;
    CK(cudaSetDevice(h->device));
    size_t n2 = (size_t)h->nbf * h->nbf;
    if (!h->dJ || !h->dK || !h->dD) {
        if ((rc = dalloc(h, &h->dJ, n2)) || (rc = dalloc(h, &h->dK, n2)) || (rc = dalloc(h, &h->dD, n2))) return rc;
    }
    size_t cin = (size_t)h->nbf * std::max(ldc, 1), uin = (size_t)h->nbf * std::max(ldu, 1);
    size_t need = std::max(cin, uin);
    if (need > h->dCin_elems) {
        h->dCin_elems = 0;
        if ((rc = dalloc(h, &h->dCin, need)) || (rc = dalloc(h, &h->dCrin, need))) return rc;
        h->dCin_elems = need;
    }
    cudaStream_t s = h->stream;
    if (nocc > 0) CK(cudaMemcpyAsync(h->dCin, C, cin * 8, cudaMemcpyHostToDevice, s));
    if (nu > 0) CK(cudaMemcpyAsync(h->dCrin, U, uin * 8, cudaMemcpyHostToDevice, s));
    if ((rc = enqueue_incremental(h, h->dCin, nocc, ldc, h->dCrin, nu, npos, ldu, mode, h->dJ, h->dK))) return rc;
    if (mode & GDFJK_DO_K) CK(cudaMemcpyAsync(K, h->dK, n2 * 8, cudaMemcpyDeviceToHost, s));
    if (mode & GDFJK_DO_J) CK(cudaMemcpyAsync(J, h->dJ, n2 * 8, cudaMemcpyDeviceToHost, s));
    if ((rc = wait_stream(h, env_timeout()))) return rc;
    return check_device_flag(h);
}

int gdfjk_compute_incremental_device(gdfjk_t h, const double* C, int nocc, int ldc, const double* U, int nu, int npos,
                                     int ldu, int mode, double* J, double* K) {
    int rc = check_incremental_args(h, C, nocc, ldc, U, nu, npos, ldu, mode, J, K);
    if (rc) return rc;
    CK(cudaSetDevice(h->device));
    return enqueue_incremental(h, C, nocc, ldc, U, nu, npos, ldu, mode, J, K);
}

int gdfjk_synchronize(gdfjk_t h, double timeout_s) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "synchronize: null handle");
    CK(cudaSetDevice(h->device));
    int rc = wait_stream(h, timeout_s);
    if (rc) return rc;
    return check_device_flag(h);
}

int gdfjk_backward(gdfjk_t h, const double* C, int nocc, int ldc, const double* gJ, const double* gK, double* dC,
                   double* Gamma, int on_device) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "backward: null handle");
    if (!h->B_ready) return set_err(h, GDFJK_ERR_STATE, "backward: B has not been uploaded");
    if (nocc < 0 || (nocc > 0 && (!C || ldc < nocc)) || !gJ || !gK)
        return set_err(h, GDFJK_ERR_ARG, "backward: bad C / nocc / ldc or null gradients");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int nbf = h->nbf, nbf_pad = h->nbf_pad, naux = h->naux;
    const int nocc_pad = round_up(std::max(nocc, 0), 32);
    int rc = ensure_workspace(h, std::max(nocc_pad, 32), false, true);
    if (rc == GDFJK_ERR_OOM) {  // as the native K: release the tensor-core forms' copies of B, retry once
        CK(cudaStreamSynchronize(s));
        mixed_release(h->mixed);
        oz_release(h->oz);
        rc = ensure_workspace(h, std::max(nocc_pad, 32), false, true);
    }
    if (rc) return rc;
    size_t np2 = (size_t)nbf_pad * nbf_pad, n2 = (size_t)nbf * nbf;
    size_t npair = (size_t)nbf * (nbf + 1) / 2;
    if (!h->gJp || !h->gKp || !h->Jg || !h->gq || !h->Dw2 || !h->Jgt) {
        if ((rc = dalloc(h, &h->gJp, np2)) || (rc = dalloc(h, &h->gKp, np2)) || (rc = dalloc(h, &h->Jg, np2)) ||
            (rc = dalloc(h, &h->gq, (size_t)naux)) || (rc = dalloc(h, &h->Dw2, (size_t)std::max(h->ntiles, 1) * TILE_ELEMS)) ||
            (rc = dalloc(h, &h->Jgt, (size_t)std::max(h->ntiles, 1) * TILE_ELEMS)))
            return rc;
    }
    if (nocc_pad > h->bw_cap_nocc) {
        h->bw_cap_nocc = -1;
        int nqb = back_transform_qblocks(naux);
        if ((rc = dalloc(h, &h->Yb, (size_t)nbf_pad * naux * nocc_pad)) ||
            (rc = dalloc(h, &h->Zpart, (size_t)nqb * nbf_pad * nocc_pad)) ||
            (rc = dalloc(h, &h->dCp, (size_t)nbf_pad * nocc_pad)))
            return rc;
        h->bw_cap_nocc = nocc_pad;
    }
    const double *dC_in = C, *dgJ = gJ, *dgK = gK;
    double *dC_out = dC, *dG = Gamma;
    if (!on_device) {
        // host-buffer path: stage through device copies sized for this call
        if ((rc = dalloc(h, &h->hC, (size_t)nbf * std::max(ldc, 1))) || (rc = dalloc(h, &h->hgJ, n2)) ||
            (rc = dalloc(h, &h->hgK, n2)) || (rc = dalloc(h, &h->hdC, (size_t)nbf * std::max(nocc, 1))))
            return rc;
        if (Gamma && (rc = dalloc(h, &h->hG, (size_t)naux * npair))) return rc;
        if (nocc > 0) CK(cudaMemcpyAsync(h->hC, C, (size_t)nbf * ldc * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->hgJ, gJ, n2 * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->hgK, gK, n2 * 8, cudaMemcpyHostToDevice, s));
        dC_in = h->hC;
        dgJ = h->hgJ;
        dgK = h->hgK;
        dC_out = dC ? h->hdC : nullptr;
        dG = Gamma ? h->hG : nullptr;
    }
    TileLayout L = layout_of(h);
    // forward pieces: padded C, D, d_Q, X
    if (nocc_pad > 0) launch_pad_C(dC_in, nbf, nocc, ldc, nbf_pad, nocc_pad, h->Cl, s);
    launch_density(h->Cl, h->Cl, nbf_pad, nocc_pad, h->D, s);
    launch_weighted_density_tiles(h->D, nbf_pad, L, h->Dw, s);
    launch_j_pass1(h->B, h->Dw, naux, L, h->dq, s);
    // g_Q = sum B_Q,mn gJ_mn
    launch_pad_sym(dgJ, nbf, nbf_pad, h->gJp, s);
    launch_pad_sym(dgK, nbf, nbf_pad, h->gKp, s);
    launch_weighted_density_tiles(h->gJp, nbf_pad, L, h->Dw2, s);
    launch_j_pass1(h->B, h->Dw2, naux, L, h->gq, s);
    if (nocc_pad > 0) {
        launch_k_transform_fp64(h->B, h->Cl, naux, nbf_pad, nocc_pad, L, h->Xl, s);
        // Y = gK X   (X viewed as nbf_pad x (naux*nocc_pad))
        size_t kd = (size_t)naux * nocc_pad;
        launch_gemm_nn_fp64(nbf_pad, kd, nbf_pad, h->gKp, nbf_pad, h->Xl, kd, 1.0, 0.0, h->Yb, kd, s);
    }
    if (dG) {
        CK(cudaMemsetAsync(dG, 0, (size_t)naux * npair * 8, s));
        if (nocc_pad > 0)
            launch_gamma(h->Yb, h->Cl, h->gJp, h->D, h->dq, h->gq, naux, nbf, nbf_pad, nocc_pad, L, dG, s);
    }
    if (dC_out && nocc > 0) {
        // J[gJ] = sum_Q B_Q g_Q (dense, padded)
        launch_j_pass2(h->B, h->gq, naux, L, h->Jgt, s);
        CK(cudaMemsetAsync(h->Jg, 0, np2 * 8, s));
        launch_unpack_tiles(h->Jgt, L, nbf, nbf_pad, h->Jg, nbf_pad, true, s);
        // Z = sum_Q B_Q Y_Q  (fixed-order reduction over Q blocks), dC = 2 Z + 2 J[gJ] C
        launch_back_transform_fp64(h->B, h->Yb, naux, nbf_pad, nocc_pad, L, h->Zpart, s);
        int nqb = back_transform_qblocks(naux);
        int qper = (naux + nqb - 1) / nqb;
        nqb = (naux + qper - 1) / qper;
        launch_reduce_blocks(h->Zpart, nqb, (size_t)nbf_pad * nocc_pad, 2.0, 0.0, h->dCp, s);
        launch_gemm_nn_fp64(nbf_pad, nocc_pad, nbf_pad, h->Jg, nbf_pad, h->Cl, nocc_pad, 2.0, 1.0, h->dCp, nocc_pad, s);
        launch_copy_rect(h->dCp, nbf, nocc, nocc_pad, dC_out, on_device ? ldc : nocc, s);
    }
    CK(cudaGetLastError());
    if (!on_device) {
        if (dC && nocc > 0) CK(cudaMemcpyAsync(dC, h->hdC, (size_t)nbf * nocc * 8, cudaMemcpyDeviceToHost, s));
        if (Gamma) CK(cudaMemcpyAsync(Gamma, h->hG, (size_t)naux * npair * 8, cudaMemcpyDeviceToHost, s));
        if ((rc = wait_stream(h, env_timeout()))) return rc;
        return check_device_flag(h);
    }
    return GDFJK_OK;
}

int gdfjk_backward_gamma_device(gdfjk_t h, const double* C, int nocc, int ldc, const double* gJ, const double* gK,
                                const int64_t* col_map, int64_t ldg, double* Gamma, int batch_q) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "backward_gamma: null handle");
    if (!h->B_ready) return set_err(h, GDFJK_ERR_STATE, "backward_gamma: B has not been uploaded");
    const int nbf = h->nbf, nbf_pad = h->nbf_pad, naux = h->naux;
    const size_t npair = (size_t)nbf * (nbf + 1) / 2;
    if (nocc <= 0 || !C || ldc < nocc || !gJ || !gK || !Gamma || batch_q < 0 ||
        ldg < (int64_t)(col_map ? 1 : npair))
        return set_err(h, GDFJK_ERR_ARG, "backward_gamma: bad C / nocc / ldc / ldg or null argument");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int nocc_pad = round_up(nocc, 32);
    int rc = ensure_workspace(h, nocc_pad, false, false);
    if (rc) return rc;
    const size_t np2 = (size_t)nbf_pad * nbf_pad;
    if (!h->gJp || !h->gKp || !h->Jg || !h->gq || !h->Dw2 || !h->Jgt) {
        if ((rc = dalloc(h, &h->gJp, np2)) || (rc = dalloc(h, &h->gKp, np2)) || (rc = dalloc(h, &h->Jg, np2)) ||
            (rc = dalloc(h, &h->gq, (size_t)naux)) || (rc = dalloc(h, &h->Dw2, (size_t)std::max(h->ntiles, 1) * TILE_ELEMS)) ||
            (rc = dalloc(h, &h->Jgt, (size_t)std::max(h->ntiles, 1) * TILE_ELEMS)))
            return rc;
    }
    // aux batch: X_b and Y_b (nbf_pad x qb x nocc_pad each) within GDFJK_BW_BATCH_GB (default 16 GB)
    const double per_q = 2.0 * nbf_pad * nocc_pad * 8.0;
    int qb = batch_q;
    if (qb == 0) {
        const char* e = getenv("GDFJK_BW_BATCH_GB");
        double gb = e ? atof(e) : 16.0;
        if (!(gb > 0.0)) gb = 16.0;
        qb = (int)std::max(1.0, std::floor(gb * 1e9 / per_q));
    }
    qb = std::max(1, std::min({qb, naux, 65535}));
    // Gamma_Q = Y_Q C^T + C Y_Q^T (+ the Coulomb terms) as P = Y_Q C^T on the tensor cores for
    // sub-batches of qs aux functions (P within GDFJK_BW_GAMMA_GB, default 8 GB), then a gather
    // of the listed pairs: those of the stored tiles (m >= n) that Gamma keeps
    int qs;
    {
        const char* e = getenv("GDFJK_BW_GAMMA_GB");
        double gb = e ? atof(e) : 8.0;
        if (!(gb > 0.0)) gb = 8.0;
        qs = (int)std::max(1.0, std::floor(gb * 1e9 / ((double)nbf_pad * nbf_pad * 8.0)));
        qs = std::min(qs, qb);
    }
    std::vector<int> pm, pn, pcol;
    {
        std::vector<int64_t> cm;
        if (col_map) {
            cm.resize(npair);
            CK(cudaMemcpy(cm.data(), col_map, npair * sizeof(int64_t), cudaMemcpyDeviceToHost));
        }
        for (int t = 0; t < h->ntiles; ++t) {
            const int I = h->tI[t], J = h->tJ[t];
            for (int r = 0; r < TILE; ++r)
                for (int c = 0; c < TILE; ++c) {
                    const int m = I * TILE + r, n = J * TILE + c;
                    if (m >= nbf || n >= nbf || m < n) continue;
                    const size_t tri = (size_t)m * (m + 1) / 2 + n;
                    const int64_t col = col_map ? cm[tri] : (int64_t)tri;
                    if (col < 0) continue;
                    pm.push_back(m);
                    pn.push_back(n);
                    pcol.push_back((int)col);
                }
        }
    }
    double *Xb = nullptr, *Yb = nullptr, *Yq = nullptr, *Pq = nullptr;
    int *d_pm = nullptr, *d_pn = nullptr, *d_pcol = nullptr;
    auto release = [&]() {
        void* ps[] = {Xb, Yb, Yq, Pq, d_pm, d_pn, d_pcol};
        for (void* p : ps)
            if (p) cudaFree(p);
        Xb = Yb = Yq = Pq = nullptr;
        d_pm = d_pn = d_pcol = nullptr;
    };
    const size_t be = (size_t)nbf_pad * qb * nocc_pad;
    const size_t npl = pm.size();
    if ((rc = dalloc(h, &Xb, be)) || (rc = dalloc(h, &Yb, be)) ||
        (rc = dalloc(h, &Yq, (size_t)qs * nbf_pad * nocc_pad)) || (rc = dalloc(h, &Pq, (size_t)qs * nbf_pad * nbf_pad)) ||
        (rc = dalloc(h, &d_pm, std::max<size_t>(npl, 1))) || (rc = dalloc(h, &d_pn, std::max<size_t>(npl, 1))) ||
        (rc = dalloc(h, &d_pcol, std::max<size_t>(npl, 1)))) {
        release();
        return rc;
    }
    if (npl > 0 && (cudaMemcpy(d_pm, pm.data(), npl * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
                    cudaMemcpy(d_pn, pn.data(), npl * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
                    cudaMemcpy(d_pcol, pcol.data(), npl * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)) {
        release();
        return set_err(h, GDFJK_ERR_CUDA, "backward_gamma: copy of the pair list failed");
    }
    TileLayout L = layout_of(h);
    launch_pad_C(C, nbf, nocc, ldc, nbf_pad, nocc_pad, h->Cl, s);
    launch_density(h->Cl, h->Cl, nbf_pad, nocc_pad, h->D, s);
    launch_weighted_density_tiles(h->D, nbf_pad, L, h->Dw, s);
    launch_j_pass1(h->B, h->Dw, naux, L, h->dq, s);
    launch_pad_sym(gJ, nbf, nbf_pad, h->gJp, s);
    launch_pad_sym(gK, nbf, nbf_pad, h->gKp, s);
    launch_weighted_density_tiles(h->gJp, nbf_pad, L, h->Dw2, s);
    launch_j_pass1(h->B, h->Dw2, naux, L, h->gq, s);
    if (cudaMemsetAsync(Gamma, 0, (size_t)naux * ldg * 8, s) != cudaSuccess) {
        release();
        return set_err(h, GDFJK_ERR_CUDA, "backward_gamma: clearing Gamma failed");
    }
    if (!h->oz) h->oz = oz_create();
    for (int q0 = 0; q0 < naux; q0 += qb) {
        const int nq = std::min(qb, naux - q0);
        const size_t kd = (size_t)nq * nocc_pad;
        // X_b[m][Q][i] = sum_n B_Q,mn C_ni over this batch's rows of B
        launch_k_transform_fp64(h->B + (size_t)q0 * h->ntiles * TILE_ELEMS, h->Cl, nq, nbf_pad, nocc_pad, L, Xb, s);
        // Y_b = gK X_b on the tensor cores (the metric contraction's FP64-accurate digit product)
        rc = oz_gemm(h->oz, h->gKp, (size_t)nbf_pad, Xb, kd, Yb, kd, nbf_pad, (int)kd, nbf_pad, 0, s, h->err);
        if (rc) {
            release();
            return set_err(h, rc, "backward_gamma: " + h->err);
        }
        for (int qs0 = 0; qs0 < nq; qs0 += qs) {
            const int nqs = std::min(qs, nq - qs0);
            launch_y_to_qmajor(Yb, nq, qs0, nqs, nbf_pad, nocc_pad, Yq, s);
            rc = oz_gemm(h->oz, Yq, (size_t)nocc_pad, h->Cl, (size_t)nocc_pad, Pq, (size_t)nbf_pad, nqs * nbf_pad, nbf_pad,
                         nocc_pad, 0, s, h->err, 1);
            if (rc) {
                release();
                return set_err(h, rc, "backward_gamma: " + h->err);
            }
            launch_gamma_gather(Pq, nqs, nbf_pad, d_pm, d_pn, d_pcol, npl, h->gJp, h->D, h->dq + q0 + qs0,
                                h->gq + q0 + qs0, Gamma + (size_t)(q0 + qs0) * ldg, (size_t)ldg, s);
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    release();
    if (e != cudaSuccess) return set_err(h, GDFJK_ERR_CUDA, std::string("backward_gamma: ") + cudaGetErrorString(e));
    return check_device_flag(h);
}

int gdfjk_debug_refuse_allocations(int after, int count) {
    if (after < 0 || count < 0) return set_err(nullptr, GDFJK_ERR_ARG, "debug_refuse_allocations: negative count");
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    const long pending = g_alloc_refuse;
    g_alloc_pass = after;
    g_alloc_refuse = count;
    return (int)std::min<long>(pending, 1 << 30);
}

int gdfjk_debug_wait_probe(gdfjk_t h, double limit_s) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "wait_probe: null handle");
    if (!(limit_s > 0.0) || limit_s > 10.0) return set_err(h, GDFJK_ERR_ARG, "wait_probe: limit must be in (0, 10] s");
    CK(cudaSetDevice(h->device));
    int rc = mixed_wait_probe(h->mixed, (unsigned long long)(limit_s * 1e9), h->stream, h->err);
    if (rc) return set_err(h, rc, h->err);
    if ((rc = wait_stream(h, env_timeout()))) return rc;
    return check_device_flag(h);
}

int gdfjk_trim(gdfjk_t h) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "trim: null handle");
    CK(cudaSetDevice(h->device));
    int rc = wait_stream(h, env_timeout());
    if (rc) return rc;
    mixed_release(h->mixed);
    oz_release(h->oz);
    return GDFJK_OK;
}

int gdfjk_last_timings(gdfjk_t h, double* j_ms, double* kt_ms, double* kc_ms) {
    if (!h) return set_err(h, GDFJK_ERR_ARG, "last_timings: null handle");
    float a = 0, b = 0, c = 0;
    CK(cudaEventSynchronize(h->ev[4]));
    CK(cudaEventElapsedTime(&a, h->ev[0], h->ev[1]));
    CK(cudaEventElapsedTime(&b, h->ev[2], h->ev[3]));
    CK(cudaEventElapsedTime(&c, h->ev[3], h->ev[4]));
    if (h->last_emulated) {
        // batches interleave transform and contraction: report the transform kernels' own time
        // and the rest of K (digits of C, splits, contractions, reductions) as the contraction
        const float k_all = b + c;
        b = oz_last_transform_ms(h->oz);
        c = k_all - b;
    }
    if (j_ms) *j_ms = a;
    if (kt_ms) *kt_ms = b;
    if (kc_ms) *kc_ms = c;
    return GDFJK_OK;
}

}  // extern "C"
