// rbg_static.cu -- a pricing entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host process that reserved all of
// the GPU's memory for its own pool at start-up and forbids libraries from
// allocating behind its back, or a latency-critical pricing loop that must
// not take cudaMalloc's implicit device-wide synchronisation on the hot
// path.  rbg_price_rt_static serves them.  It runs the same mixed-form
// kernels as rbg_price_rt (fused Philox + Volterra + variance kernel, FP32
// payoffs, FP64 merges), but all of its scratch lives in one file-scope
// __device__ array of kStaticScratchBytes (16 MiB), which every GPU that
// loads this library holds until the process exits.
//
// The device address of that array is looked up once per device, with the
// device current, on the first call on that device (cudaGetSymbolAddress).
// The address stays cached for the life of the process, so a cudaDeviceReset
// between calls is not supported.  Every call synchronises its stream to
// return the prices, so none can run under stream capture.  All calls share the array and it keeps
// the last call's contents; what must start at zero (the kernel error word
// and the running sums) is cleared by every call.  Calls whose work overlaps
// on the GPU race on the array, so callers serialise them (one stream, or
// their own ordering).  A call that fails after it has queued work waits for
// that work before it returns, so the next call never meets it on the array.
//
// The results equal rbg_price_rt's: the same batch size B and paths per
// payoff thread G where the buffers fit; where they do not, B is cut to a
// smaller whole number of 256 G-path payoff chunks, so every path is summed
// in the same FP32 chunk as in rbg_price_rt and only the order of the FP64
// merges of whole chunks changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "rbg_internal.hpp"
#include "rbg_mixed.hpp"

namespace rbg {

constexpr size_t kStaticScratchBytes = (size_t)16 << 20;
constexpr int kStaticMaxDevices = 64;
constexpr int kStaticMaxOutputs = 4096;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static std::mutex g_static_mu;
static void* g_static_ptr[kStaticMaxDevices] = {nullptr};
static thread_local std::string g_static_err;

static int static_fail(int code, const std::string& msg)
{
    g_static_err = msg;
    return code;
}

// Device address of the scratch array on the current device (set-up once).
static int static_scratch(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return static_fail(RBG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= kStaticMaxDevices) return static_fail(RBG_ERR_UNSUPPORTED, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_static_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return static_fail(RBG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        }
        g_static_ptr[dev] = ptr;
    }
    *out = g_static_ptr[dev];
    return RBG_OK;
}

static size_t up256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace rbg

using namespace rbg;

extern "C" {

const char* rbg_static_last_error(void) { return g_static_err.c_str(); }

size_t rbg_static_scratch_bytes(void) { return kStaticScratchBytes; }

int rbg_price_rt_static(const rbg_params* p, const rbg_options* o, double* price, double* stat, double* iv)
{
    if (!p || !o || !price || !stat) return static_fail(RBG_ERR_ARG, "null params/options/outputs");
    if (o->precision != RBG_MIXED) return static_fail(RBG_ERR_UNSUPPORTED, "the static entry point runs the mixed form");
    Plan plan;
    std::string err;
    if (!build_plan(*p, plan, err)) return static_fail(RBG_ERR_ARG, err);
    const int n_out = (int)plan.outs.size();
    if (n_out > kStaticMaxOutputs)
        return static_fail(RBG_ERR_ARG, "par_size * op_size exceeds 4096 outputs of the static scratch");
    MixedJob job;
    // the two-pass kernel without the A-tile cache, which would not fit the static scratch
    int rc = mixed_prepare(plan, *o, p->M, job, err, 0, false, false);
    if (rc) return static_fail(rc, err);

    // carve the scratch: workspace image, output tables, sums, results,
    // chunk partials, then the per-batch (Ivdt, IsvdW) buffer
    const size_t off_ws = 0;
    const size_t off_outs = up256(off_ws + job.workspace_bytes);
    const size_t off_T = up256(off_outs + sizeof(OutDev) * n_out);
    const size_t off_acc = up256(off_T + sizeof(double) * n_out);
    const size_t off_res = up256(off_acc + sizeof(double) * 4 * n_out);
    const size_t off_part = up256(off_res + sizeof(double) * 5 * n_out);
    if (off_part >= kStaticScratchBytes)
        return static_fail(RBG_ERR_ARG, "tables of this job exceed the 16 MiB static scratch");
    // batch B and paths per payoff thread G as rbg_price_rt chooses them; if
    // the (Ivdt, IsvdW) buffer and partials do not fit, B is halved and cut
    // down to whole payoff chunks of 256 G paths, G kept.  Fused jobs need no
    // (Ivdt, IsvdW) buffer and one partial row per CTA.
    int64_t B = std::min<int64_t>(p->M, job.batch);
    const int G = payoff_paths_per_thread(B, job.sms);
    const int64_t chunk = 256 * (int64_t)G;
    int64_t nchunk_max = 1;
    size_t off_ivb = 0;
    for (;;) {
        nchunk_max = job.fused ? mixed_part_rows(job, B) : (B + chunk - 1) / chunk;
        off_ivb = up256(off_part + (size_t)32 * n_out * nchunk_max);
        const size_t ivb_bytes = job.fused ? 0 : (size_t)8 * plan.vgs.size() * B;
        if (off_ivb + ivb_bytes <= kStaticScratchBytes) break;
        if (job.fused || B <= chunk)
            return static_fail(RBG_ERR_ARG, "variance groups / outputs of this job exceed the static scratch");
        B = std::max<int64_t>(chunk, (B / 2) / chunk * chunk);
    }
    void* base = nullptr;
    if ((rc = static_scratch(&base))) return rc;
    unsigned char* s = (unsigned char*)base;
    // a null stream means the calling thread's per-thread default stream, which
    // does not synchronise with the other streams of the process as the legacy
    // default stream would
    cudaStream_t st = o->stream ? (cudaStream_t)o->stream : cudaStreamPerThread;
    // error exits once work is queued: let that work finish first, so that the
    // caller's next call does not race it on the shared array
    auto fail_queued = [&](int code, const std::string& msg) {
        cudaStreamSynchronize(st);
        cudaGetLastError();
        return static_fail(code, msg);
    };

    std::vector<OutDev> outs(n_out);
    std::vector<double> Tv(n_out);
    for (int i = 0; i < n_out; ++i) {
        outs[i] = OutDev{plan.outs[i].rho, plan.outs[i].K, plan.outs[i].vg, 0};
        Tv[i] = plan.outs[i].T;
    }
    cudaError_t e = cudaMemcpyAsync(s + off_ws, job.host_ws.data(), job.host_ws.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s + off_outs, outs.data(), sizeof(OutDev) * n_out, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s + off_T, Tv.data(), sizeof(double) * n_out, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s + off_acc, 0, sizeof(double) * 4 * n_out, st);
    if (e != cudaSuccess) return fail_queued(RBG_ERR_CUDA, std::string("static scratch upload: ") + cudaGetErrorString(e));
    for (int64_t m0 = 0; m0 < p->M; m0 += B) {
        const int64_t b = std::min(B, p->M - m0);
        if (job.fused) {
            const int rows = mixed_part_rows(job, b);
            e = cudaMemsetAsync(s + off_part, 0, (size_t)32 * n_out * rows, st);
            if (e != cudaSuccess)
                return fail_queued(RBG_ERR_CUDA, std::string("static scratch clear: ") + cudaGetErrorString(e));
            rc = mixed_launch(job, s + off_ws, o->seed, o->path_offset + m0, b, nullptr, st, err, nullptr, nullptr,
                              (double*)(s + off_part));
            if (rc) return fail_queued(rc, err);
            launch_accumulate((const double*)(s + off_part), rows, n_out, (double*)(s + off_acc), st);
            continue;
        }
        rc = mixed_launch(job, s + off_ws, o->seed, o->path_offset + m0, b, s + off_ivb, st, err);
        if (rc) return fail_queued(rc, err);
        const int nchunks = (int)((b + chunk - 1) / chunk);
        launch_payoff_sums_f32((const OutDev*)(s + off_outs), n_out, s + off_ivb, b, G, (double*)(s + off_part),
                               nchunks, st);
        launch_accumulate((const double*)(s + off_part), nchunks, n_out, (double*)(s + off_acc), st);
    }
    launch_finalize((const double*)(s + off_acc), n_out, p->M, (const OutDev*)(s + off_outs),
                    (const double*)(s + off_T), o->compute_iv, (double*)(s + off_res), st);
    // the error word after the finalize is queued: one wait for the whole call
    if ((rc = mixed_check(job, s + off_ws, st, err))) return fail_queued(rc, err);
    std::vector<double> res(5 * (size_t)n_out);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(res.data(), s + off_res, sizeof(double) * 5 * n_out, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_queued(RBG_ERR_CUDA, std::string("static pricing: ") + cudaGetErrorString(e));
    std::memcpy(price, res.data(), sizeof(double) * n_out);
    std::memcpy(stat, res.data() + n_out, sizeof(double) * n_out);
    if (iv) std::memcpy(iv, res.data() + 2 * n_out, sizeof(double) * n_out);
    return RBG_OK;
}

}  // extern "C"
