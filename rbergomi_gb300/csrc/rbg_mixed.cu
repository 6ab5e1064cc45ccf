// rbg_mixed.cu -- the mixed-precision form of the RT pricer on sm_103a.
//
// One persistent kernel per Volterra pass (distinct H) fuses
//   Philox4x32-10 normals (FP32 Box-Muller) for W1 and W1perp,
//   the hybrid-scheme convolution Y2[p][j] = sum_{k<j} W1[p][k] Gamma[j-k]
//     as a block-lower-triangular Toeplitz GEMM on the tcgen05 tensor cores
//     (BF16x3 or FP16x3 split products, FP32 accumulation in TMEM),
//   the variance path v and the Romano-Touzi integrals
//     Ivdt = dt sum v, IsvdW = sum sqrt(v) sdt W1   (FP32, per variance group)
// and writes one float2 per (variance group, path).  A second kernel prices
// every (rho, K) output in FP32 and reduces across paths in FP64.
//
// Arithmetic restated from rBergLib/rBergomiMT.cpp:73-109 (updateV,
// updateWtilde), :163-167 (scaleWtilde), :427-436 (intVdt, intRootVdW) and
// :598-602 (the conditional BS payoff).
//
// Toeplitz structure.  Time steps are cut into K-chunks of 32.  Chunk c
// multiplies the A tile W1[:, 32c, 32c+32) into output columns [32c, Np):
//   D[:, 32c + j'] += sum_{k'<32} A_c[:, k'] * S[j'][k'],  S[j'][k'] = Gamma[j' - k'],
// and S does not depend on c.  So one Np x 32 strip S (hi and lo halves,
// 64 KB at N = 512) stays resident in shared memory for the whole kernel,
// loaded once by a bulk async copy; only A tiles stream.  Two-pass tiles
// (below) use a narrow strip instead: the two K = 16 halves of a chunk read
// the same 16-wide P[r][k''] = Gamma[r - 16 - k''] at row offsets 16 apart,
// (Np + 16) x 16 (65 KB at N = 1024).  After chunk c's MMAs, columns
// [32c, 32c+32) are final and the epilogue reads them.
//
// TMEM holds 128 lanes x 512 FP32 columns.  For Np > 512 a tile runs np =
// ceil(Np / 512) passes: pass 0 accumulates columns [0, 32 n0), n0 = (Np -
// 512 (np - 1)) / 32, from chunks 0 .. n0-1; every later pass accumulates the
// next 512 columns, first from the A tiles of all earlier chunks drawn again
// (W1 only, no epilogue work), then from its own chunks.  For two passes the
// producers' chunk sequence per tile is
//   [0, n0) real | [0, n0) redrawn | [n0, nc) real.
// For the 16-bit splits and the RT estimator on Philox normals, 512 < Np <=
// 1024 runs pass mode 3 instead (PassPlan): 256-column passes alternating
// between two TMEM buffers, each chunk drawn once, the far-field of the next
// pass accumulated in the other buffer from the chunks' A tiles that the MMA
// thread keeps in a per-CTA global cache; its epilogue reads W1 back from the
// A tile (hi + lo), so a stage holds no FP32 W1 tile and three stages fit.
// Up to Np = 1024 the whole narrow strip stays in shared memory.  Above that
// (up to 4096, eight passes) only its first 528 rows do -- all that a chunk
// drawn for real reads -- and each redrawn chunk brings the 528-row window it
// reads into its stage's FP32-tile region by a bulk copy (33 KB, from L2).
//
// Warp roles (544 threads, 576 in the multi-pass modes; one CTA per SM,
// persistent over 128-path tiles):
//   warps 0-7   producers, two threads per path, 16 steps each per chunk:
//               Philox -> FP32 normals; W1 split into hi/lo 16-bit A tiles
//               (SW64 K-major layout); FP32 W1, W1perp kept for the epilogue
//   warps 8-15  epilogue, two warpgroups (16 accumulator columns each per
//               chunk), one TMEM lane quadrant per warp: tcgen05.ld,
//               X = Y2 + a1 W1 + a2 W1perp, v and the two integrals
//   warp 16     TMEM allocation and the single-thread tcgen05.mma issuer
//   warp 17     multi-pass modes only: a second issuing thread on another
//               scheduler (one 256-column TMEM half, or pass mode 3's
//               far-field), as one thread competing for issue slots with
//               sixteen arithmetic warps held the multi-pass pipeline
// Every mbarrier wait is bounded (%globaltimer); on expiry the kernel records
// an error word, drains its MMAs, frees TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <mutex>

#include "rbg_device.cuh"
#include "rbg_mixed.hpp"

namespace rbg {

constexpr int kTileM = 128;
constexpr int kChunk = 32;
constexpr int kMaxG = kMixedMaxGroups;
#ifndef RBG_PROD_WARPS
#define RBG_PROD_WARPS 8
#endif
#ifndef RBG_EPI_WARPS
#define RBG_EPI_WARPS 8
#endif
#ifndef RBG_FUSE_PAYOFFS
#define RBG_FUSE_PAYOFFS 0
#endif
#ifndef RBG_PASS3
#define RBG_PASS3 1  // pass mode 3 for the two-pass range where it applies (0: the redrawing two-pass kernel)
#endif
constexpr int kProdWarps = RBG_PROD_WARPS;          // 4 * 128 / kProdWarps... threads per path: kProdWarps / 4
constexpr int kEpiWarps = RBG_EPI_WARPS;            // 4 (one warpgroup) or 8 (two, 16 columns each per chunk)
constexpr int kEpiWGs = kEpiWarps / 4;
constexpr int kStepsPerThread = kChunk * 4 / kProdWarps;  // producer steps per chunk per thread
constexpr int kEpiWarp0 = kProdWarps;               // warps 8..15: TMEM lane quadrant = warp % 4
constexpr int kMmaWarp = kProdWarps + kEpiWarps;    // warp 16
constexpr int kThreads = (kMmaWarp + 1) * 32;       // 544
constexpr int kPassCols = 512;                      // TMEM: 128 lanes x 512 FP32 columns per pass
constexpr int kMaxNp = 2 * kPassCols;               // two passes with the whole narrow strip resident
constexpr int kMaxNpMulti = 8 * kPassCols;          // up to eight passes with streamed strip windows
constexpr int kStripK = 16;                         // narrow strip width: one K = 16 MMA step
// Pass mode 3 (below): 256-column passes in two TMEM buffers, and slots for
// the cached A tiles the far-field MMAs read.
constexpr int kHalfCols = kPassCols / 2;
constexpr int kCSlots = 3;
constexpr int kHPerPath = kProdWarps * 32 / kTileM; // producer threads per path
constexpr uint64_t kWaitNs = 2000000000ull;         // 2 s per wait

// shared-memory layout (offsets from a 1024-aligned base):
//   [strip hi | strip lo]            2 * Np * 64 B, SW64 (one pass), or 2 * (Np + 16) * 32 B, SW32
//   A tiles, per stage [hi | lo]     16 KB per stage (1024-aligned)
//   FP32 tiles, per stage            w1 [128][32], w1perp [128][32] (swizzled), W1 of step P0 [128]
//   per-thread group sums            n_g * 2 * 128 floats
//   beta tables                      n_g * Np floats
//   fused outputs                    table n_o * 4 floats, FP32 Kahan sums [4 warps][n_o][4]
//   mbarriers + TMEM address
constexpr int kTileBytes = kTileM * kChunk * 2;                          // one 16-bit 128 x 32 tile, 8 KB
constexpr int kStageA = 2 * kTileBytes;                                  // hi + lo
// FP32 stage: W1 tile, W1perp tile, W1 boundary row; plain Monte Carlo adds
// a Wperp tile and its boundary row (offsets in floats)
constexpr int kFW1p = kChunk * kTileM, kFBnd = 2 * kChunk * kTileM, kFWq = kFBnd + kTileM;
constexpr int kFWqBnd = kFWq + kChunk * kTileM;
__host__ __device__ constexpr int stage_f_bytes(int ns) { return (ns == 3 ? kFWqBnd + kTileM : kFWq) * 4; }

// Strip width in K: the full chunk (32, SW64 rows, one row per output
// column) where one TMEM pass covers Np; 16 (SW32, 16 leading zero rows)
// for two-pass tiles, whose Np-row strip would not fit shared memory at 32.
__host__ __device__ inline int strip_k(int Np) { return Np <= kPassCols ? kChunk : kStripK; }
// Pass mode of a tile: 0 one TMEM pass, 1 two passes over the resident
// narrow strip, 2 up to eight passes where only the strip's first
// kWindowRows rows stay resident and the chunks drawn again for a later pass
// bring their strip window into shared memory by bulk copy.
__host__ __device__ inline int pass_mode(int Np) { return Np <= kPassCols ? 0 : (Np <= kMaxNp ? 1 : 2); }
// Narrow-strip rows one pass of one chunk reads: 512 columns + 16 (K halves).
constexpr int kWindowRows = kPassCols + kStripK;
constexpr int kWindowBytes = kWindowRows * kStripK * 2;  // one 16-bit half, 16896 B
// TF32 split (split kind 2): the strip is always narrow, P[r][k] = Gamma[r -
// 24 - k], Np + 24 rows of 8 FP32 (32 B, SW32); the four K = 8 steps of a
// chunk read it at row offsets 8 apart.  Its window is 512 + 24 rows.
constexpr int kStripKT = 8;
constexpr int kLeadT = kChunk - kStripKT;                   // 24 leading zero rows
constexpr int kWindowRowsT = kPassCols + kLeadT;            // 536
constexpr int kWindowBytesT = kWindowRowsT * kStripKT * 4;  // one TF32 half, 17152 B
// Kernel split kind of an rbg_split: 0 FP16x3, 1 BF16x3, 2 TF32x2.
inline int split_kind(int split) { return split == RBG_SPLIT_BF16X3 ? 1 : (split == RBG_SPLIT_F16X3 ? 0 : 2); }
// FP32 tiles are path-major, [128 paths][32 steps], with the 16-byte chunk
// index XORed by (path mod 8): a thread's 4 consecutive steps are one vector
// access and the 8 threads of a vector phase hit distinct banks.
__device__ __forceinline__ int ftile_at(int p, int s) { return p * kChunk + ((((s >> 2) ^ (p & 7))) << 2) + (s & 3); }

__host__ __device__ inline int strip_bytes(int Np)
{
    return strip_k(Np) == kChunk ? 2 * Np * kChunk * 2 : 2 * (Np + kStripK) * kStripK * 2;
}

struct SmemLayout {
    int strip, a0, f0, fstride, stages, cs, acc, beta, otab, osum, bars, total;
};

__host__ __device__ inline int strip_bytes_t32(int Np) { return 2 * (Np + kLeadT) * kStripKT * 4; }
__host__ __device__ inline int strip_bytes_sk(int Np, bool tf32) { return tf32 ? strip_bytes_t32(Np) : strip_bytes(Np); }

// Resident strip bytes: the whole image (pass modes 0, 1) or the first
// kWindowRows rows of each half (pass mode 2).
__host__ __device__ inline int strip_smem_bytes(int Np)
{
    return pass_mode(Np) == 2 ? 2 * kWindowBytes : strip_bytes(Np);
}
__host__ __device__ inline int strip_smem_bytes_t32(int Np)
{
    return pass_mode(Np) == 2 ? 2 * kWindowBytesT : strip_bytes_t32(Np);
}

// ns: normal streams per path, 2 (RT) or 3 (plain Monte Carlo: ns sums per group).
// In pass mode 2 a stage's FP32-tile region also holds a redrawn chunk's strip
// window (hi and lo halves), so it is at least 2 kWindowBytes (a multiple of
// the 256-byte SW32 swizzle atom).
// tf32: the TF32 strip geometry (split kind 2).
// cslots: pass mode 3's slots for cached A tiles (1024-aligned, after the FP32
// tiles; 0 in the other pass modes, whose layout it leaves unchanged).
__host__ __device__ inline SmemLayout smem_layout(int Np, int stages, int n_g, int n_o, int ns = 2, bool tf32 = false,
                                                  int cslots = 0)
{
    SmemLayout L;
    L.strip = 0;
    L.a0 = ((tf32 ? strip_smem_bytes_t32(Np) : strip_smem_bytes(Np)) + 1023) / 1024 * 1024;
    L.stages = stages;
    L.f0 = L.a0 + stages * kStageA;
    // pass mode 3 (cslots > 0) keeps only the W1perp tile: W1 is read back from the stage's A tile
    L.fstride = cslots > 0 ? kChunk * kTileM * 4 : stage_f_bytes(ns);
    const int win2 = tf32 ? 2 * kWindowBytesT : 2 * kWindowBytes;
    if (pass_mode(Np) == 2 && L.fstride < win2) L.fstride = win2;
    L.cs = L.f0 + stages * L.fstride;
    if (cslots > 0) L.cs = (L.cs + 1023) / 1024 * 1024;
    L.acc = L.cs + cslots * kStageA;
    // per warpgroup, then W1_0 (Wperp_0), then (pass mode 3) the deferred sqrt(v) per group
    L.beta = L.acc + 2 * n_g * ns * kTileM * 4 + (ns - 1) * kTileM * 4 + (cslots > 0 ? n_g * kTileM * 4 : 0);
    L.otab = L.beta + n_g * Np * 4;
    L.osum = (L.otab + n_o * 16 + 15) / 16 * 16;
    L.bars = L.osum + kEpiWarps * n_o * 16;
    L.total = L.bars + (cslots > 0 ? 256 : 128) + 1024;  // barriers + alignment slack for the dynamic base
    return L;
}

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Adds `bytes` to the phase's expected transaction count without arriving.
__device__ __forceinline__ void mbar_expect_tx_only(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Bulk copy global -> shared memory of this CTA (16-byte aligned addresses,
// a multiple of 16 bytes), completing `bytes` transactions on `bar`.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Bulk copy shared memory of this CTA -> global (16-byte aligned addresses, a
// multiple of 16 bytes) as one bulk async-group of the issuing thread.
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// The issuing thread's bulk stores: every source read (read0), every store
// complete (done0), or all but the most recent one complete (done1).
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_done0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_done1() { asm volatile("cp.async.bulk.wait_group 1;" ::: "memory"); }

// One wait attempt; the hardware may suspend the thread for up to 20 us
// (the suspend-time hint) until the phase completes, so waiting warps do not
// spin on the issue slots the working roles need.
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(20000u)
        : "memory");
    return ok != 0;
}

// Non-blocking test of a phase.
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of the given parity; false on timeout or when
// another role already failed (then the caller winds down).  The error word
// and the clock are polled every 64 tries only (at most 64 x 20 us apart).  With `prof` set (diagnostic
// runs), lane 0 adds the cycles it waited to prof[site].  LIMIT_NS: the time
// limit, a compile-time constant (2 s in the pricing kernels).
template <uint64_t LIMIT_NS = kWaitNs>
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned int* err, unsigned int site,
                                       unsigned long long* prof = nullptr)
{
    if (mbar_try(bar, parity)) return true;
    const long long c0 = prof ? clock64() : 0;
    const uint64_t t0 = globaltimer();
    bool ok = true;
    for (uint32_t it = 1;; ++it) {
        if (mbar_try(bar, parity)) break;
        if ((it & 63u) == 0u) {
            if (*(volatile unsigned int*)err != 0u) { ok = false; break; }
            if (globaltimer() - t0 > LIMIT_NS) {
                atomicCAS(err, 0u, site);
                ok = false;
                break;
            }
        }
    }
    if (prof && (threadIdx.x & 31) == 0) atomicAdd(prof + site, (unsigned long long)(clock64() - c0));
    return ok;
}

// Waits up to 10 ms for a phase whatever the error word says: a CTA winding
// down after an error lets its own bulk copies in flight land before it exits.
__device__ __noinline__ void mbar_drain(uint32_t bar, uint32_t parity)
{
    const uint64_t t0 = globaltimer();
    while (!mbar_try(bar, parity) && globaltimer() - t0 < 10000000ull) {
    }
}

// the same wait, made warp-uniform so .sync.aligned tcgen05 ops stay converged;
// the first try is inline, so a phase that has already completed (the common
// case in a balanced pipeline) costs no call
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity, unsigned int* err, unsigned int site,
                                               unsigned long long* prof = nullptr)
{
    const bool ok = mbar_try(bar, parity) || mbar_wait(bar, parity, err, site, prof);
    return __all_sync(0xffffffffu, ok);
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// SW64 K-major shared-memory matrix descriptor (tcgen05 format): start
// address >> 4, LBO (unused for swizzled K-major) = 1, SBO = 8 rows x 64 B,
// version bit 46, layout type SWIZZLE_64B (4) in bits 61-63.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

// SW32 K-major descriptor for the 16-wide strip: 32-byte rows, SBO = 8 rows
// x 32 B, layout type SWIZZLE_32B (6).
__device__ __forceinline__ uint64_t sdesc_sw32(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(256 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)6 << 61);
}

// SW128 K-major descriptor for the TF32 A tile: 128-byte rows (32 FP32), SBO
// = 8 rows x 128 B, layout type SWIZZLE_128B (2).  A K = 8 step starts 32 B
// further into the row; the tile base is 1024-aligned, so the swizzle phase
// (address bits 7-9, the row) is unchanged and the base offset stays 0.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32 (2), both K-major.
__device__ __forceinline__ uint32_t idesc_tf32(int n)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

// FP32 -> TF32 rounded to nearest even (the low 13 bits of the result are 0).
__device__ __forceinline__ uint32_t tf32_rn(float x)
{
    uint32_t r;
    asm("cvt.rn.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16 (1) or F16 (0),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ uint32_t idesc_f16(int n, int ab_bf16)
{
    const uint32_t fmt = ab_bf16 ? 1u : 0u;
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// The three split products of one chunk's 16-bit A tile (hi at ahi, lo
// 8 KB above) against the narrow strip (hi / lo halves at bhi / blo) into n
// TMEM columns from d, the first of which reads strip row jrow (K half ks
// from row jrow + 16 - 16 ks).  overwrite: the first product replaces D.
//
// One thread issues every MMA of the CTA while sixteen warps of Philox and
// epilogue arithmetic compete for its issue slots (in isolation the MMA pipe
// takes 144 cycles per N = 256 MMA in this pattern, 183 beside eight such
// warps), so the descriptors are formed with one 32-bit add each: a chunk's
// descriptors differ only in the start-address field, address >> 4 in bits
// 0-13 of the low word, and shared addresses stay below 2^18, so adding an
// offset / 16 never carries out of it.
__device__ __forceinline__ uint64_t sdesc_words(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }

template <int SK>
__device__ __forceinline__ void mma_chunk_narrow(uint32_t d, uint32_t ahi, uint32_t bhi, uint32_t blo, uint32_t jrow,
                                                 int n, bool overwrite)
{
    const uint32_t id = idesc_f16(n, SK);
    const uint64_t a0 = sdesc_sw64(ahi), b0 = sdesc_sw32(bhi + jrow * (kStripK * 2));
    const uint32_t alo = (uint32_t)a0, ahw = (uint32_t)(a0 >> 32), blo0 = (uint32_t)b0, bhw = (uint32_t)(b0 >> 32);
    const uint32_t dl = (blo - bhi) >> 4;  // hi half -> lo half of the strip (or window)
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        // A: K half ks 32 B into the row, lo tile kTileBytes above; B: rows from jrow + 16 - 16 ks
        const uint64_t dah = sdesc_words(alo + 2u * ks, ahw), dal = sdesc_words(alo + kTileBytes / 16 + 2u * ks, ahw);
        const uint32_t bro = (uint32_t)(kStripK * (1 - ks) * kStripK * 2 / 16);
        const uint64_t dbh = sdesc_words(blo0 + bro, bhw), dbl = sdesc_words(blo0 + dl + bro, bhw);
        umma_f16(d, dah, dbh, id, (overwrite && ks == 0) ? 0u : 1u);
        umma_f16(d, dah, dbl, id, 1u);
        umma_f16(d, dal, dbh, id, 1u);
    }
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Split kinds of the mixed-form convolution: 0 FP16x3, 1 BF16x3 (A and B
// each split into 16-bit hi + lo, three products), 2 TF32 with one
// compensation term (A rounded to TF32, B = hi + lo in TF32, two products).
// 16-bit split x = hi + lo (+ O(2^-16 |x|) for BF16, O(2^-22 |x|) for FP16)
template <int BF16>
__device__ __forceinline__ void split2(float x0, float x1, uint32_t& hi, uint32_t& lo)
{
    if (BF16) {
        __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
        float2 hf = __bfloat1622float2(h);
        __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
        hi = *reinterpret_cast<uint32_t*>(&h);
        lo = *reinterpret_cast<uint32_t*>(&l);
    } else {
        __half2 h = __floats2half2_rn(x0, x1);
        float2 hf = __half22float2(h);
        __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
        hi = *reinterpret_cast<uint32_t*>(&h);
        lo = *reinterpret_cast<uint32_t*>(&l);
    }
}

// One element (path row p, step k of the chunk) of the A tile: hi / lo
// 16-bit halves in SW64 rows of 64 B, or (SK = 2) one TF32 in SW128 rows of
// 128 B.
template <int SK>
__device__ __forceinline__ void a_tile_store1(unsigned char* st, int p, int k, float z)
{
    if constexpr (SK == 2) {
        const int off = p * 128 + ((((k >> 2)) ^ (p & 7)) << 4) + ((k & 3) << 2);
        *(uint32_t*)(st + off) = tf32_rn(z);
    } else {
        uint32_t hi, lo;
        split2<SK>(z, 0.f, hi, lo);
        const int off = p * 64 + ((((k >> 3)) ^ ((p >> 1) & 3)) << 4) + ((k & 7) << 1);
        *(unsigned short*)(st + off) = (unsigned short)hi;
        *(unsigned short*)(st + kTileBytes + off) = (unsigned short)lo;
    }
}

// W1 of path row p read back from a 16-bit A tile as hi + lo (the operand
// the tensor cores multiply; within 2^-18 |W1| of the FP32 draw for BF16,
// 2^-22 for FP16): steps [16 hh, 16 hh + 16) of the chunk, or step k.
template <int SK>
__device__ __forceinline__ float2 split_pair_f32(uint32_t w)
{
    if constexpr (SK == 1) {
        return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xFFFF0000u));
    } else {
        __half2 h;
        *reinterpret_cast<uint32_t*>(&h) = w;
        return __half22float2(h);
    }
}
template <int SK>
__device__ __forceinline__ void a_tile_w1_16(const unsigned char* st, int p, int hh, float (&w)[16])
{
    const int sw = (p >> 1) & 3;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const int off = p * 64 + (((2 * hh + e) ^ sw) << 4);
        const uint4 h = *(const uint4*)(st + off), l = *(const uint4*)(st + kTileBytes + off);
        const uint32_t hv[4] = {h.x, h.y, h.z, h.w}, lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 a = split_pair_f32<SK>(hv[i]), b = split_pair_f32<SK>(lv[i]);
            w[8 * e + 2 * i] = a.x + b.x;
            w[8 * e + 2 * i + 1] = a.y + b.y;
        }
    }
}
template <int SK>
__device__ __forceinline__ float a_tile_w1_at(const unsigned char* st, int p, int k)
{
    const int off = p * 64 + ((((k >> 3)) ^ ((p >> 1) & 3)) << 4) + (((k & 7) >> 1) << 2);
    const float2 a = split_pair_f32<SK>(*(const uint32_t*)(st + off)),
                 b = split_pair_f32<SK>(*(const uint32_t*)(st + kTileBytes + off));
    return (k & 1) ? a.y + b.y : a.x + b.x;
}

// --------------------------------------------------------------- the kernel
// Conditional BS call (tau = 1, r = 0) from (Ivdt, IsvdW) in FP32
// (rBergLib/rBergomiMT.cpp:598-602 with BlackScholes.cpp:16-21).  ITM strikes
// go through put-call parity, (S - K) + put, so both wings are computed from
// small tail probabilities that keep their relative accuracy.
// The strike-independent part: conditional spot, log-spot, vol and 1 / vol.
struct RtSpot {
    float lnS, spot, rv, vol;
    bool deg;  // zero conditional variance: the payoff is intrinsic
};

__device__ __forceinline__ RtSpot rt_spot_f32(float Ivdt, float IsvdW, float rho)
{
    RtSpot r;
    const float v2 = (1.0f - rho * rho) * Ivdt;
    r.lnS = -0.5f * rho * rho * Ivdt + rho * IsvdW;
    r.spot = ex2_approx(1.4426950408889634f * r.lnS);
    r.deg = !(v2 > 0.0f);
    r.rv = rsqrt_approx(v2);
    r.vol = v2 * r.rv;
    return r;
}

// Without a branch on the money side: paths of one warp fall on both sides
// of a near-the-money strike, and a branch there made the warp evaluate both
// sides' two normal CDFs (23 % of the payoff kernel's time).  The side only
// flips the CDFs' arguments; the expressions are the branching form's below,
// so the bits are the same.
__device__ __forceinline__ float rt_payoff_f32(const RtSpot& r, float K, float lnK)
{
    const float d1 = fmaf(r.lnS - lnK, r.rv, 0.5f * r.vol);
    const float d2 = d1 - r.vol;
    const bool itm = r.spot > K;
    const float p1 = phi_f32(itm ? -d1 : d1), p2 = phi_f32(itm ? -d2 : d2);
    const float v = itm ? (r.spot - K) + (K * p2 - r.spot * p1) : r.spot * p1 - K * p2;
    return r.deg ? fmaxf(r.spot - K, 0.0f) : v;
}

// The branching form, for the path kernel's fused-payoff epilogue: the
// branch-free one there moved that kernel's code generation by 0.15 % even
// though ordinary launches never run the fused loop.
__device__ __forceinline__ float rt_payoff_f32(float Ivdt, float IsvdW, float rho, float K, float lnK)
{
    const RtSpot r = rt_spot_f32(Ivdt, IsvdW, rho);
    if (r.deg) return fmaxf(r.spot - K, 0.0f);
    const float d1 = fmaf(r.lnS - lnK, r.rv, 0.5f * r.vol);
    const float d2 = d1 - r.vol;
    if (r.spot > K) return (r.spot - K) + (K * phi_f32(-d2) - r.spot * phi_f32(-d1));
    return r.spot * phi_f32(d1) - K * phi_f32(d2);
}

// One producer thread's share of a chunk: Philox -> FP32 normals for steps
// [32 c + SPT h, + SPT) of path p, its hi/lo row of the A tile and, unless
// REDRAW (a first-pass chunk drawn again for the second pass), the FP32 W1 /
// W1perp tiles the epilogue reads.  Compiled per REDRAW so that the W1 and
// W1perp Philox streams stay interleaved in the common case.
// FW1 = false (pass mode 3): no FP32 W1 tile, W1perp at the start of the
// stage's FP32 region (the epilogue reads W1 back from the A tile).
template <int SK, bool REDRAW, bool MC, bool FW1 = true>
__device__ __forceinline__ void produce_chunk(const MixedArgs& a, const PhiloxKeys& keys, uint64_t gpath, bool valid,
                                              int64_t m, int p, int h, int c, bool bnd, unsigned char* st,
                                              float* w1s)
{
    constexpr int SPT = kStepsPerThread;
    const int Np = a.Np;
    const int sw = (p >> 1) & 3;
    float* w1ps = w1s + kFW1p;
    const int step0 = kChunk * c + SPT * h;
    float w[SPT], wp[SPT], wq[MC ? SPT : 1];
#pragma unroll
    for (int q = 0; q < SPT / 4; ++q) {
        const uint32_t g = (uint32_t)((step0 >> 2) + q);
        const uint4 x0 = philox_group(keys, gpath, g, 0);
        box_muller_f32(x0.x, x0.y, w[4 * q], w[4 * q + 1]);
        box_muller_f32(x0.z, x0.w, w[4 * q + 2], w[4 * q + 3]);
        if (!REDRAW) {
            const uint4 x1 = philox_group(keys, gpath, g, 1);
            box_muller_f32(x1.x, x1.y, wp[4 * q], wp[4 * q + 1]);
            box_muller_f32(x1.z, x1.w, wp[4 * q + 2], wp[4 * q + 3]);
        }
        if (MC && !REDRAW) {  // plain Monte Carlo: Wperp on stream 2
            const uint4 x2 = philox_group(keys, gpath, g, 2);
            box_muller_f32(x2.x, x2.y, wq[4 * q], wq[4 * q + 1]);
            box_muller_f32(x2.z, x2.w, wq[4 * q + 2], wq[4 * q + 3]);
        }
    }
    if (!(valid && step0 + SPT <= a.N)) {  // only the last tile / chunk
#pragma unroll
        for (int q = 0; q < SPT; ++q) {
            if (!valid || step0 + q >= a.N) {
                w[q] = 0.f;
                wp[q] = 0.f;
                if (MC) wq[q] = 0.f;
            }
        }
    }
    if constexpr (SK == 2) {
        // A tile: row p, 128 B of TF32 (rounded to nearest), 16-byte chunks covering
        // steps [SPT h, SPT h + SPT), SW128 swizzle (chunk XOR row mod 8)
#pragma unroll
        for (int e = 0; e < SPT / 4; ++e) {
            const int off = p * 128 + ((((SPT / 4) * h + e) ^ (p & 7)) << 4);
            *(uint4*)(st + off) = make_uint4(tf32_rn(w[4 * e]), tf32_rn(w[4 * e + 1]), tf32_rn(w[4 * e + 2]),
                                             tf32_rn(w[4 * e + 3]));
        }
    } else {
        // A tile: row p, logical 16-byte chunks covering steps [SPT h, SPT h + SPT), SW64 swizzle
        uint32_t hi[SPT / 2], lo[SPT / 2];
#pragma unroll
        for (int q = 0; q < SPT / 2; ++q) split2<SK>(w[2 * q], w[2 * q + 1], hi[q], lo[q]);
#pragma unroll
        for (int e = 0; e < SPT / 8; ++e) {
            const int off = p * 64 + ((((SPT / 8) * h + e) ^ sw) << 4);
            *(uint4*)(st + off) = make_uint4(hi[4 * e], hi[4 * e + 1], hi[4 * e + 2], hi[4 * e + 3]);
            *(uint4*)(st + kTileBytes + off) = make_uint4(lo[4 * e], lo[4 * e + 1], lo[4 * e + 2], lo[4 * e + 3]);
        }
    }
    if (!REDRAW) {
#pragma unroll
        for (int q = 0; q < SPT; q += 4) {
            const int at = ftile_at(p, SPT * h + q);
            if (FW1) {
                *(float4*)(w1s + at) = make_float4(w[q], w[q + 1], w[q + 2], w[q + 3]);
                *(float4*)(w1ps + at) = make_float4(wp[q], wp[q + 1], wp[q + 2], wp[q + 3]);
            } else {
                *(float4*)(w1s + at) = make_float4(wp[q], wp[q + 1], wp[q + 2], wp[q + 3]);
            }
            if (MC) *(float4*)(w1s + kFWq + at) = make_float4(wq[q], wq[q + 1], wq[q + 2], wq[q + 3]);
        }
        // last real chunk of a pass that is not the last: its successor (chunk
        // c + 1) follows the next pass's redrawn chunks, so W1 at step 32 (c + 1)
        // for the last column's sqrt(v) dW goes into this stage's boundary row
        if (bnd && h == kHPerPath - 1) {
            const uint4 xb = philox_group(keys, gpath, (uint32_t)(8 * (c + 1)), 0);
            float b0, b1;
            box_muller_f32(xb.x, xb.y, b0, b1);
            w1s[kFBnd + p] = valid ? b0 : 0.f;
            if (MC) {
                const uint4 xq = philox_group(keys, gpath, (uint32_t)(8 * (c + 1)), 2);
                box_muller_f32(xq.x, xq.y, b0, b1);
                w1s[kFWqBnd + p] = valid ? b0 : 0.f;
            }
        }
        if (a.dbg_w && valid) {
#pragma unroll
            for (int q = 0; q < SPT; ++q) {
                a.dbg_w[(m * 2 + 0) * Np + step0 + q] = w[q];
                a.dbg_w[(m * 2 + 1) * Np + step0 + q] = wp[q];
            }
        }
    }
}

// Sobol' producer (RT, rbg_price_rt_sobol in the mixed form): warp w of the
// producers draws paths 16 w .. 16 w + 15 of the tile and lane l step
// j = 32 c + l, i.e. coordinates 2 j (W1) and 2 j + 1 (W1perp) of the
// paths' points path0 + m + 1 (rBergomi/rBergomiMT.cpp:669-670 with breakZ).
// The first point comes from its Gray code, the next 15 by one XOR each
// (point s + 1 = point s ^ v[ctz(s + 1)]).  a.sob holds bits 30..61 of the
// direction integers, [32][2N] uint32 (point indices below 2^32).  Table
// reads are issued independently of the XORs that use them: the Gray-code
// rows as one unrolled predicated batch, and the walk's rows up front (15
// consecutive indices have ctz <= 3 except at most one multiple of 16).
// Writes the FP32 W1 / W1perp tiles and the 16-bit hi/lo A tile (REDRAW: W1
// and the A tile only).

// The Gray-code start: XOR of the table rows of the set bits of g (< 2^KB),
// all loads issued before the XORs need them.
template <int KB>
__device__ __forceinline__ void sobol_gray_start(const uint2* tab, int N, int j, unsigned long long g,
                                                 unsigned int& q0, unsigned int& q1)
{
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        if ((g >> k) & 1ull) {
            const uint2 v = __ldg(tab + (size_t)k * N + j);
            q0 ^= v.x;
            q1 ^= v.y;
        }
    }
}

// One point of the Sobol' producer: lane's step j of path row p (path m),
// from the point's coordinates q0 (W1) and q1 (W1perp).
template <int SK, bool REDRAW>
__device__ __forceinline__ void sobol_point(const MixedArgs& a, int p, int64_t m, int j, int lane, bool jin,
                                            unsigned int q0, unsigned int q1, unsigned char* st, float* w1s)
{
    const bool ok = jin && m < a.B;
    const float z0 = ok ? sobol_normal_f32(q0) : 0.f;
    const float z1 = (ok && !REDRAW) ? sobol_normal_f32(q1) : 0.f;
    if (!REDRAW) {
        const int at = ftile_at(p, lane);
        w1s[at] = z0;
        w1s[kFW1p + at] = z1;
        if (a.dbg_w && m < a.B) {
            a.dbg_w[(m * 2 + 0) * a.Np + j] = z0;
            a.dbg_w[(m * 2 + 1) * a.Np + j] = z1;
        }
    }
    a_tile_store1<SK>(st, p, lane, z0);
}

template <int SK, bool REDRAW>
__device__ __forceinline__ void produce_chunk_sobol(const MixedArgs& a, int64_t tile, int c, bool bnd, unsigned char* st,
                                                    float* w1s)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int N = a.N;
    const int j = kChunk * c + lane;
    const bool jin = j < N;
    const int64_t m0 = tile * kTileM + 16 * w;
    const unsigned long long s0 = (unsigned long long)(a.path0 + m0) + 1ull;
    const uint2* tab = reinterpret_cast<const uint2*>(a.sob);  // [32][N] coordinate pairs
    unsigned int q0 = 0, q1 = 0;
    uint2 r[4] = {}, rb = {};  // the walk's rows 0..3 and the row of the one multiple of 16 in (s0, s0 + 15]
    const unsigned long long m16 = ((s0 >> 4) + 1) << 4;
    const bool has16 = m16 <= s0 + 15;
    if (jin) {
        const unsigned long long g = s0 ^ (s0 >> 1);  // point indices stay below 2^32
        if ((g >> 20) == 0ull)  // warp-uniform: fewer than 2^20 points in
            sobol_gray_start<20>(tab, N, j, g, q0, q1);
        else
            sobol_gray_start<32>(tab, N, j, g, q0, q1);
#pragma unroll
        for (int k = 0; k < 4; ++k) r[k] = __ldg(tab + (size_t)k * N + j);
        if (has16) rb = __ldg(tab + (size_t)(__ffsll((long long)m16) - 1) * N + j);
    }
    if ((s0 & 15ull) == 1ull) {
        // s0 = 16 t + 1 (path offsets that are multiples of 16): s0 + i + 1 =
        // 16 t + i + 2, so the walk's rows are fixed by i -- 1, 0, 2, 0, 1, 0, 3,
        // 0, 1, 0, 2, 0, 1, 0 and the multiple of 16 last
#pragma unroll 1
        for (int t = 0; t < 4; ++t) {
            const int i0 = 4 * t, p0 = 16 * w + i0;
            sobol_point<SK, REDRAW>(a, p0, m0 + i0, j, lane, jin, q0, q1, st, w1s);
            q0 ^= r[1].x; q1 ^= r[1].y;
            sobol_point<SK, REDRAW>(a, p0 + 1, m0 + i0 + 1, j, lane, jin, q0, q1, st, w1s);
            q0 ^= r[0].x; q1 ^= r[0].y;
            sobol_point<SK, REDRAW>(a, p0 + 2, m0 + i0 + 2, j, lane, jin, q0, q1, st, w1s);
            const uint2 v = t == 1 ? r[3] : t == 3 ? rb : r[2];
            q0 ^= v.x; q1 ^= v.y;
            sobol_point<SK, REDRAW>(a, p0 + 3, m0 + i0 + 3, j, lane, jin, q0, q1, st, w1s);
            q0 ^= r[0].x; q1 ^= r[0].y;
        }
    } else {
#pragma unroll 4
        for (int i = 0; i < 16; ++i) {
            sobol_point<SK, REDRAW>(a, 16 * w + i, m0 + i, j, lane, jin, q0, q1, st, w1s);
            if (i < 15) {
                const int k = __ffsll((long long)(s0 + i + 1)) - 1;
                const uint2 v = k == 0 ? r[0] : k == 1 ? r[1] : k == 2 ? r[2] : k == 3 ? r[3] : rb;
                q0 ^= v.x;
                q1 ^= v.y;
            }
        }
    }
    // last real chunk of a pass before the last: W1 at step 32 (c + 1) for the boundary row
    if (!REDRAW && bnd && lane < 16) {
        const int p = 16 * w + lane, jb = kChunk * (c + 1);
        const unsigned long long sb = s0 + lane;
        unsigned int q = 0;
        for (unsigned long long g = sb ^ (sb >> 1); g; g &= g - 1)
            q ^= __ldg(a.sob + (size_t)(__ffsll((long long)g) - 1) * 2 * N + 2 * jb);
        w1s[kFBnd + p] = (m0 + lane < a.B && jb < N) ? sobol_normal_f32(q) : 0.f;
    }
}

// Caller-normals producer (the mixed quadrature entry points): the caller's
// FP64 normals in the quadrature layout, path m's stream s at a.ext +
// (m NS + s) N.  Warp w of the producers takes paths 16 w .. 16 w + 15 of the
// tile and lane l step j = 32 c + l, so each load instruction reads 32
// consecutive doubles of one row (256 B, coalesced; no alignment beyond the
// doubles' own).  Writes the FP32 W1 / W1perp (/ Wperp) tiles and the 16-bit
// hi/lo A tile (REDRAW: W1 and the A tile only).
template <int SK, bool REDRAW, bool MC>
__device__ __forceinline__ void produce_chunk_ext(const MixedArgs& a, int64_t tile, int c, bool bnd, unsigned char* st,
                                                  float* w1s)
{
    constexpr int NS = MC ? 3 : 2;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int N = a.N, Np = a.Np;
    const int j = kChunk * c + lane;
    const bool jin = j < N;
    const int64_t m0 = tile * kTileM + 16 * w;
    float* w1ps = w1s + kFW1p;
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
        const int p = 16 * w + i;
        const int64_t m = m0 + i;
        const bool ok = jin && m < a.B;
        const double* z = a.ext + (size_t)m * NS * N + j;
        const float z0 = ok ? (float)__ldg(z) : 0.f;
        if (!REDRAW) {
            w1s[ftile_at(p, lane)] = z0;
            w1ps[ftile_at(p, lane)] = ok ? (float)__ldg(z + N) : 0.f;
            if (MC) w1s[kFWq + ftile_at(p, lane)] = ok ? (float)__ldg(z + 2 * N) : 0.f;
            if (a.dbg_w && m < a.B) {
                a.dbg_w[(m * 2 + 0) * Np + j] = z0;
                a.dbg_w[(m * 2 + 1) * Np + j] = w1ps[ftile_at(p, lane)];
            }
        }
        a_tile_store1<SK>(st, p, lane, z0);
    }
    // the next chunk's rows into L2 while this one is consumed: the loads above
    // keep too few bytes in flight to cover HBM latency on their own.  One
    // 128-byte line per 16 lanes; every address stays inside its row.
    if ((lane & 15) == 0 && j + kChunk < N) {
#pragma unroll 4
        for (int i = 0; i < 16; ++i) {
            if (m0 + i >= a.B) break;
            const double* z = a.ext + (size_t)(m0 + i) * NS * N + j + kChunk;
#pragma unroll
            for (int s = 0; s < (REDRAW ? 1 : NS); ++s)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(z + (size_t)s * N));
        }
    }
    // last real chunk of a pass before the last: W1 (and Wperp) at step 32 (c + 1)
    // for the boundary rows
    if (!REDRAW && bnd && lane < 16) {
        const int p = 16 * w + lane;
        const int64_t m = m0 + lane;
        const double* z = a.ext + (size_t)m * NS * N + kChunk * (c + 1);
        w1s[kFBnd + p] = m < a.B ? (float)__ldg(z) : 0.f;
        if (MC) w1s[kFWqBnd + p] = m < a.B ? (float)__ldg(z + 2 * N) : 0.f;
    }
}

// Pass schedule of a tile.  TMEM holds 512 accumulator columns, so a tile of
// Np > 512 columns runs np passes: pass 0 covers chunks [0, n0) (columns
// [0, 32 n0), n0 = (Np - 512 (np - 1)) / 32), pass p >= 1 the 16 chunks from
// pass_begin(p) = n0 + 16 (p - 1).  Pass p takes chunks 0 .. pass_end(p) - 1 in
// order: those below pass_begin(p) are drawn again (W1 only) and add their
// whole contribution to the pass's columns; the rest are drawn for real and
// their columns become final one chunk at a time, as in one pass.  Every role
// walks this same (pass, chunk) sequence, one pipeline stage per chunk.
//
// Pass mode 3 cuts the columns into passes of 256 (pass 0: n0 chunks, the
// rest 8 each) held alternately in two TMEM buffers, and draws every chunk
// once.  While pass q's own chunks accumulate into its buffer and its columns
// are read, the other buffer takes the next pass's whole far-field: each of
// pass q's chunks over all 256 next-pass columns, and every earlier chunk
// (0 .. begin(q) - 1) from a per-CTA global cache of A tiles that the MMA
// thread stored when the chunk was first used.  So the far-field MMAs overlap
// the producers' work instead of waiting for redrawn tiles, and a pass's
// columns are complete when its first own chunk lands.
template <int PM>
struct PassPlan {
    static constexpr int kPer = (PM == 3 ? kHalfCols : kPassCols) / kChunk;  // chunks of a pass after the first
    int np, n0, nc;
    __device__ __forceinline__ PassPlan(const MixedArgs& a)
        : np(PM == 0 ? 1 : (PM == 1 ? 2 : a.np)), n0(PM == 0 ? 0 : a.n0), nc(a.nc) {}
    __device__ __forceinline__ int begin(int p) const { return p == 0 ? 0 : n0 + kPer * (p - 1); }
    __device__ __forceinline__ int end(int p) const { return p + 1 >= np ? nc : n0 + kPer * p; }
};

// PM: pass mode (pass_mode(Np)): 0 one TMEM pass; 1 two passes, the narrow
// strip resident; 2 up to eight passes, the strip's first window of rows
// resident and each redrawn chunk's window brought into its stage's FP32-tile
// region by a bulk copy that the stage's `full` barrier waits for.
// SRC: where the normals come from: 0 Philox, 1 Sobol' (produce_chunk_sobol,
// RT only), 2 the caller's FP64 normals (a.ext, quadrature layout).
// SK: split kind (0 FP16x3, 1 BF16x3, 2 TF32 with one compensation term).
template <int SK, int PM, bool MC, int SRC = 0>
__global__ void __launch_bounds__(PM > 0 ? kThreads + 32 : kThreads, 1) k_mixed_gemm(const __grid_constant__ MixedArgs a)
{
    constexpr int NS = MC ? 3 : 2;  // normal streams per path = sums per variance group
    constexpr int kStageFB = stage_f_bytes(NS);
    constexpr bool T32 = SK == 2;
    constexpr int WB = T32 ? kWindowBytesT : kWindowBytes;  // one half of a strip window
    static_assert(PM >= 0 && PM <= 3 && SK >= 0 && SK <= 2, "pass mode / split kind");
    static_assert(PM != 3 || (SK != 2 && !MC && SRC == 0), "pass mode 3: 16-bit splits, RT, Philox");
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const SmemLayout L = smem_layout(a.Np, a.stages, a.n_g, a.n_o, NS, T32, PM == 3 ? kCSlots : 0);
    unsigned char* strip = base + L.strip;
    float* acc_s = (float*)(base + L.acc);
    float* beta_s = (float*)(base + L.beta);
    float4* otab = (float4*)(base + L.otab);   // (rho, K, lnK, local group) per fused output
    float* osum = (float*)(base + L.osum);     // [epilogue warp][output][S, C, S2, C2], FP32 Kahan
    uint64_t* bars = (uint64_t*)(base + L.bars);
    // barrier slots
    const int S = a.stages;
    uint64_t* full = bars;           // [S]
    uint64_t* empty = bars + 3;      // [S]
    uint64_t* accf = bars + 6;       // [S]
    uint64_t* tmem_empty = bars + 9;
    uint64_t* strip_bar = bars + 10;
    uint64_t* final_bar = bars + 11;
    uint32_t* tmem_holder = (uint32_t*)(bars + 12);
    // pass mode 3 only: the second TMEM buffer's release, the cached-tile slots' fill and release
    uint64_t* tmem_empty1 = bars + 13;
    uint64_t* cfull = bars + 14;   // [kCSlots]
    uint64_t* cempty = bars + 17;  // [kCSlots]
    uint64_t* ydone = bars + 20;   // thread 1's far-field of a pass complete

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Np = a.Np, nc = a.nc;
    const PassPlan<PM> pp(a);
    const int FB = (PM == 2 || PM == 3) ? L.fstride : kStageFB;  // bytes per stage of the FP32-tile region
    const int64_t ntiles = (a.B + kTileM - 1) / kTileM;
    const uint32_t sbytes = (uint32_t)(T32 ? strip_smem_bytes_t32(Np) : strip_smem_bytes(Np));
    const uint32_t half_g = (uint32_t)((T32 ? strip_bytes_t32(Np) : strip_bytes(Np)) / 2);  // hi -> lo in the global image

    if (threadIdx.x == kMmaWarp * 32) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_u32(full + s), kProdWarps);
            // multi-pass modes: both MMA threads commit; pass mode 3's thread 0 also arrives once the
            // A tile is in the cache
            mbar_init(smem_u32(empty + s), 1 + kEpiWarps + (PM == 3 ? 2 : (PM > 0 ? 1 : 0)));
            mbar_init(smem_u32(accf + s), 1);
        }
        mbar_init(smem_u32(tmem_empty), kEpiWarps);
        if (PM == 3) {
            mbar_init(smem_u32(tmem_empty1), kEpiWarps);
            mbar_init(smem_u32(ydone), 1);
            for (int s = 0; s < kCSlots; ++s) {
                mbar_init(smem_u32(cfull + s), 1);
                mbar_init(smem_u32(cempty + s), 1);
            }
        }
        mbar_init(smem_u32(strip_bar), 1);
        mbar_init(smem_u32(final_bar), PM > 0 ? 2 : 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(smem_u32(strip_bar), sbytes);
        if (PM == 2) {
            // the first window of each half
            bulk_g2s(smem_u32(strip), a.strip, WB, smem_u32(strip_bar));
            bulk_g2s(smem_u32(strip) + WB, a.strip + half_g, WB, smem_u32(strip_bar));
        } else {
            bulk_g2s(smem_u32(strip), a.strip, sbytes, smem_u32(strip_bar));
        }
    }
    if (warp == kMmaWarp) {
        __syncwarp();
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int i = threadIdx.x; i < a.n_g * a.Np; i += blockDim.x) beta_s[i] = a.beta[i];
    for (int i = threadIdx.x; i < a.n_o; i += blockDim.x) otab[i] = a.otab[i];
    for (int i = threadIdx.x; i < kEpiWarps * a.n_o * 4; i += blockDim.x) osum[i] = 0.f;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    const long long role_t0 = a.prof ? clock64() : 0;
    if (warp < kProdWarps) {
        // ------------------------------------------------------- producers
        const int p = threadIdx.x & (kTileM - 1);
        const int h = threadIdx.x >> 7;  // which kStepsPerThread steps of the chunk
        const PhiloxKeys keys = philox_keys(a.seed);
        // stage s and its phase parity ph run over the chunks of all tiles
        int s = 0;
        uint32_t ph = 0;
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int64_t m = tile * kTileM + p;
            const bool valid = m < a.B;
            const uint64_t gpath = (uint64_t)(a.path0 + m);
            for (int q = 0; q < pp.np; ++q) {
                const int cb = pp.begin(q), ce = pp.end(q);
                // pass mode 3 draws each chunk once: no redrawn chunks, no boundary rows
                for (int c = PM == 3 ? cb : 0; c < ce; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                    // redrawn chunks of a later pass feed only the MMA (W1 A tile)
                    const bool redraw = (PM == 1 || PM == 2) && c < cb;
                    // last real chunk of a pass before the last: boundary row for its successor
                    const bool bnd = (PM == 1 || PM == 2) && !redraw && c == ce - 1 && q + 1 < pp.np;
                    if (!mbar_wait_warp(smem_u32(empty + s), ph ^ 1u, a.err, 1, a.prof)) goto done;
                    unsigned char* st = base + L.a0 + s * kStageA;
                    float* w1s = (float*)(base + L.f0 + s * FB);
                    if (PM == 2 && redraw && threadIdx.x == 0) {
                        // this chunk's strip window, rows [32 (cb - c), + the window's rows) of each
                        // half (32-byte rows in both narrow strips), into the stage's FP32-tile
                        // region (unused by redrawn chunks); the MMA issuer's wait on `full`
                        // covers the bytes
                        const uint32_t dst = smem_u32(w1s), bar = smem_u32(full + s);
                        const unsigned char* src = a.strip + (size_t)(kChunk * (cb - c)) * 32;
                        fence_proxy_async();
                        mbar_expect_tx_only(bar, 2 * WB);
                        bulk_g2s(dst, src, WB, bar);
                        bulk_g2s(dst + WB, src + half_g, WB, bar);
                    }
                    if (SRC == 1) {
                        if (PM > 0 && redraw)
                            produce_chunk_sobol<SK, true>(a, tile, c, bnd, st, w1s);
                        else
                            produce_chunk_sobol<SK, false>(a, tile, c, bnd, st, w1s);
                    } else if (SRC == 2) {
                        if (PM > 0 && redraw)
                            produce_chunk_ext<SK, true, MC>(a, tile, c, bnd, st, w1s);
                        else
                            produce_chunk_ext<SK, false, MC>(a, tile, c, bnd, st, w1s);
                    } else if (PM == 3) {
                        produce_chunk<SK, false, MC, false>(a, keys, gpath, valid, m, p, h, c, bnd, st, w1s);
                    } else if (PM > 0 && redraw) {
                        produce_chunk<SK, true, MC>(a, keys, gpath, valid, m, p, h, c, bnd, st, w1s);
                    } else {
                        produce_chunk<SK, false, MC>(a, keys, gpath, valid, m, p, h, c, bnd, st, w1s);
                    }
                    fence_proxy_async();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(full + s));
                }
            }
        }
    } else if (warp < kMmaWarp) {
        // -------------------------------------------------------- epilogue
        const int ew = warp - kEpiWarp0;
        const int wg = ew >> 2;           // warpgroup
        const int quad = warp & 3;        // TMEM lane quadrant
        const int p = quad * 32 + lane;
        const uint32_t tlane = tmem + ((uint32_t)(quad * 32) << 16);
        // per warpgroup [group][NS sums][path]: sum v, sum sqrt(v) W1 (, sum sqrt(v) Wperp)
        float* my_acc = acc_s + (size_t)wg * a.n_g * NS * kTileM;
        float* w10_s = acc_s + (size_t)2 * a.n_g * NS * kTileM;  // W1_0 per path
        float* wq0_s = w10_s + kTileM;                          // Wperp_0 per path (plain Monte Carlo)
        // pass mode 3: per group and path, sqrt(v) of the previous chunk's last column, whose
        // dW (W1 at the next chunk's first step) is added with the next chunk
        float* pend_s = acc_s + (size_t)2 * a.n_g * NS * kTileM + (NS - 1) * kTileM;
        int s = 0;
        uint32_t ph = 0;
        int gpass = 0;  // pass mode 3: passes so far (all tiles); pass g uses TMEM buffer g & 1
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int64_t m = tile * kTileM + p;
            const bool valid = m < a.B;
            for (int g = 0; g < a.n_g; ++g)
#pragma unroll
                for (int t = 0; t < NS; ++t) my_acc[(NS * g + t) * kTileM + p] = 0.f;
            for (int q = 0; q < pp.np; ++q) {
              const int cb = pp.begin(q), ce = pp.end(q);
              for (int c = PM == 3 ? cb : 0; c < ce; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                // the producers' FP32 tiles of this stage (the upper half also pairs
                // its last column with the next chunk's first W1), then the MMA results
                if (!mbar_wait_warp(smem_u32(full + s), ph, a.err, 7, a.prof)) goto done;
                if ((PM == 1 || PM == 2) && c < cb) {
                    // redrawn chunk: no column becomes final.  Its MMA completion is still
                    // awaited, so that every accf phase is observed in order.
                    if (!mbar_wait_warp(smem_u32(accf + s), ph, a.err, 2, a.prof)) goto done;
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(empty + s));
                    continue;
                }
                // output column - TMEM column (mod 2^32); pass mode 3 alternates two 256-column buffers
                const uint32_t tcol0 = PM == 3   ? (uint32_t)(kChunk * cb) - (uint32_t)((gpass & 1) * kHalfCols)
                                       : PM > 0 ? (uint32_t)(kChunk * cb)
                                                : 0u;
                const bool pass_end = c == ce - 1;
                const bool has_next = c + 1 < nc;
                // successor W1 in this stage's boundary row (pass mode 3: the next stage holds chunk c + 1)
                const bool bnd = (PM == 1 || PM == 2) && pass_end && q + 1 < pp.np;
                const int sn = (s + 1 == S) ? 0 : s + 1;
                if (PM != 3 && (kEpiWGs == 1 || wg == 1) && has_next && !bnd &&
                    !mbar_wait_warp(smem_u32(full + sn), sn == 0 ? ph ^ 1u : ph, a.err, 8, a.prof))
                    goto done;
                if (!mbar_wait_warp(smem_u32(accf + s), ph, a.err, 2, a.prof)) goto done;
                tc_fence_after();
                const float* w1s = (const float*)(base + L.f0 + s * FB);
                const float* w1ps = PM == 3 ? w1s : w1s + kFW1p;
                const float* wqs = w1s + kFWq;  // plain Monte Carlo only
                const unsigned char* ast = base + L.a0 + s * kStageA;  // pass mode 3: W1 = hi + lo of the A tile
#pragma unroll 1
                for (int hh = wg; hh < 2; hh += kEpiWGs) {
                    const int j0 = 16 * hh;
                    // the producers' FP32 operands first: these shared-memory loads are
                    // issued ahead of the TMEM load, so their latencies overlap
                    float w1v[16], w1pv[16];
                    if constexpr (PM == 3) {
                        a_tile_w1_16<SK>(ast, p, hh, w1v);
#pragma unroll
                        for (int jj = 0; jj < 16; jj += 4) {
                            const float4 v = *(const float4*)(w1ps + ftile_at(p, j0 + jj));
                            w1pv[jj] = v.x; w1pv[jj + 1] = v.y; w1pv[jj + 2] = v.z; w1pv[jj + 3] = v.w;
                        }
                    } else {
#pragma unroll
                    for (int jj = 0; jj < 16; jj += 4) {
                        const int at = ftile_at(p, j0 + jj);
                        const float4 u = *(const float4*)(w1s + at), v = *(const float4*)(w1ps + at);
                        w1v[jj] = u.x; w1v[jj + 1] = u.y; w1v[jj + 2] = u.z; w1v[jj + 3] = u.w;
                        w1pv[jj] = v.x; w1pv[jj + 1] = v.y; w1pv[jj + 2] = v.z; w1pv[jj + 3] = v.w;
                    }
                    }
                    const float* nexts = (const float*)(base + L.f0 + sn * FB);
                    // pass mode 3: the last column's dW is added with the next chunk, when W1 at its
                    // first step (w_first) is at hand; the epilogue never waits for a later stage
                    const float w_after = (hh == 0) ? (PM == 3 ? a_tile_w1_at<SK>(ast, p, 16) : w1s[ftile_at(p, 16)])
                                                    : (PM == 3 || !has_next ? 0.f
                                                       : bnd                ? w1s[kFBnd + p]
                                                                            : nexts[ftile_at(p, 0)]);
                    const float w_first = (PM == 3 && hh == 1 && c > 0) ? a_tile_w1_at<SK>(ast, p, 0) : 0.f;
                    float wqv[MC ? 16 : 1], wq_after = 0.f;
                    if (MC) {
#pragma unroll
                        for (int jj = 0; jj < 16; jj += 4) {
                            const float4 u = *(const float4*)(wqs + ftile_at(p, j0 + jj));
                            wqv[jj] = u.x; wqv[jj + 1] = u.y; wqv[jj + 2] = u.z; wqv[jj + 3] = u.w;
                        }
                        wq_after = (hh == 0) ? wqs[ftile_at(p, 16)]
                                             : (!has_next ? 0.f
                                                : bnd     ? w1s[kFWqBnd + p]
                                                          : nexts[kFWq + ftile_at(p, 0)]);
                    }
                    float x[16];
                    tmem_ld16(tlane + (uint32_t)(kChunk * c + j0) - tcol0, x);
                    if (pass_end && hh + kEpiWGs >= 2) {
                        // this warp's accumulator columns of the pass are read
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(smem_u32((PM == 3 && (gpass & 1)) ? tmem_empty1 : tmem_empty));
                    }
                    float wn[16];
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj) {
                        const float w1 = w1v[jj];
                        x[jj] = x[jj] + a.a1 * w1 + a.a2 * w1pv[jj];
                        if (jj > 0) wn[jj - 1] = w1;
                        if (jj == 0 && j0 == 0 && c == 0) {
                            w10_s[p] = w1;
                            if (MC) wq0_s[p] = wqv[0];
                        }
                    }
                    wn[15] = w_after;
                    float wqn[MC ? 16 : 1];  // Wperp one step ahead
                    if (MC) {
#pragma unroll
                        for (int jj = 0; jj < 15; ++jj) wqn[jj] = wqv[jj + 1];
                        wqn[15] = wq_after;
                    }
                    if (a.dbg_x && valid) {
#pragma unroll
                        for (int jj = 0; jj < 16; ++jj) a.dbg_x[m * Np + kChunk * c + j0 + jj] = x[jj];
                    }
                    // v_{j+1} = xi exp(eta WS_j - comp_j): su = sqrt(v) = 2^(alpha/2 X - beta/2),
                    // one MUFU ex2 per element and group, v = su * su
                    for (int g = 0; g < a.n_g; ++g) {
                        const float ah = a.alpha[g];
                        const float* btp = beta_s + g * Np + kChunk * c + j0;
                        float bt[16];
#pragma unroll
                        for (int jj = 0; jj < 16; jj += 4) {
                            const float4 u = *(const float4*)(btp + jj);  // 16-byte aligned: Np, j0 are multiples of 16
                            bt[jj] = u.x; bt[jj + 1] = u.y; bt[jj + 2] = u.z; bt[jj + 3] = u.w;
                        }
                        const int lim = a.nsteps[g] - 1 - kChunk * c - j0;
                        float sv = 0.f, swv = 0.f, swq = 0.f, su_last = 0.f;
                        if (lim >= 16) {
#pragma unroll
                            for (int jj = 0; jj < 16; ++jj) {
                                const float su = ex2_approx(fmaf(ah, x[jj], -bt[jj]));
                                sv = fmaf(su, su, sv);
                                swv = fmaf(su, wn[jj], swv);
                                if (MC) swq = fmaf(su, wqn[jj], swq);
                                if (PM == 3 && jj == 15) su_last = su;
                            }
                        } else {
#pragma unroll
                            for (int jj = 0; jj < 16; ++jj) {
                                if (jj < lim) {
                                    const float su = ex2_approx(fmaf(ah, x[jj], -bt[jj]));
                                    sv = fmaf(su, su, sv);
                                    swv = fmaf(su, wn[jj], swv);
                                    if (MC) swq = fmaf(su, wqn[jj], swq);
                                }
                            }
                        }
                        if (PM == 3 && hh == 1) {
                            float* pg = pend_s + g * kTileM + p;
                            if (c > 0) swv = fmaf(*pg, w_first, swv);
                            *pg = su_last;
                        }
                        my_acc[(NS * g) * kTileM + p] += sv;
                        my_acc[(NS * g + 1) * kTileM + p] += swv;
                        if (MC) my_acc[(NS * g + 2) * kTileM + p] += swq;
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(empty + s));
              }
              if (PM == 3) ++gpass;
            }
            // both warpgroups' column sums of this tile are in shared memory
            asm volatile("bar.sync 1, %0;" ::"r"(kEpiWarps * 32) : "memory");
            const long long bs_t0 = a.prof ? clock64() : 0;
            const float w1_0 = w10_s[p];
            // fused payoffs: warpgroup wg prices outputs q = wg, wg + 2, ...
            // Ivdt = dt (xi + sum v), IsvdW = sdt (sqrt(xi) W1_0 + sum sqrt(v) W1)
            float iv_last = 0.f, iw_last = 0.f;
            int g_last = -1;
            for (int q = wg; q < a.n_o; q += kEpiWGs) {
                const float4 o = otab[q];
                const int g = (int)o.w;
                if (g != g_last) {
                    g_last = g;
                    float sv = acc_s[(NS * g) * kTileM + p], sw2 = acc_s[(NS * g + 1) * kTileM + p];
                    if (kEpiWGs == 2) {
                        sv += acc_s[((size_t)a.n_g * NS + NS * g) * kTileM + p];
                        sw2 += acc_s[((size_t)a.n_g * NS + NS * g + 1) * kTileM + p];
                    }
                    iv_last = a.dt[g] * (a.xi + sv);
                    iw_last = a.sdt[g] * fmaf(a.sqrt_xi, w1_0, sw2);
                }
                float x = valid ? rt_payoff_f32(iv_last, iw_last, o.x, o.y, o.z) : 0.f;
                float x2 = x * x;
#pragma unroll
                for (int sh = 16; sh > 0; sh >>= 1) {
                    x += __shfl_xor_sync(0xffffffffu, x, sh);
                    x2 += __shfl_xor_sync(0xffffffffu, x2, sh);
                }
                // warp sums in FP32, compensated (Kahan) FP32 across tiles; FP64
                // once per CTA at the end -- GB300's FP64 pipe is too slow here
                if (lane == 0) {
                    float* os = osum + ((size_t)ew * a.n_o + q) * 4;
                    kahan_add_f32(os[0], os[1], x);
                    kahan_add_f32(os[2], os[3], x2);
                }
            }
            if (wg == 0 && valid && a.ivb) {
                for (int g = 0; g < a.n_g; ++g) {
                    float sv = acc_s[(NS * g) * kTileM + p], sw2 = acc_s[(NS * g + 1) * kTileM + p];
                    if (kEpiWGs == 2) {
                        sv += acc_s[((size_t)a.n_g * NS + NS * g) * kTileM + p];
                        sw2 += acc_s[((size_t)a.n_g * NS + NS * g + 1) * kTileM + p];
                    }
                    a.ivb[(size_t)(a.g0 + g) * a.B + m] =
                        make_float2(a.dt[g] * (a.xi + sv), a.sdt[g] * fmaf(a.sqrt_xi, w1_0, sw2));
                    if (MC) {
                        // IsvdWp = sdt (sqrt(xi) Wperp_0 + sum sqrt(v_j) Wperp_j)
                        float sq = acc_s[(NS * g + 2) * kTileM + p];
                        if (kEpiWGs == 2) sq += acc_s[((size_t)a.n_g * NS + NS * g + 2) * kTileM + p];
                        a.ivq[(size_t)(a.g0 + g) * a.B + m] = a.sdt[g] * fmaf(a.sqrt_xi, wq0_s[p], sq);
                    }
                }
            }
            if (a.prof && lane == 0) atomicAdd(a.prof + 20, (unsigned long long)(clock64() - bs_t0));
            // the sums are read before either warpgroup clears its half for the next tile
            asm volatile("bar.sync 1, %0;" ::"r"(kEpiWarps * 32) : "memory");
        }
    } else if (lane == 0) {
        // ------------------------------------------------------ MMA issuer
        const uint32_t strip_hi = smem_u32(strip);
        const uint32_t strip_lo = strip_hi + (uint32_t)((T32 ? strip_smem_bytes_t32(Np) : strip_smem_bytes(Np)) / 2);
        constexpr bool wide = PM == 0 && !T32;  // the wide 16-bit strip exactly when one pass covers Np
        if constexpr (PM == 3) {
            // Pass mode 3 (PassPlan) issues its MMAs from two threads on two schedulers: one
            // thread, issuing in order, competes for issue slots with sixteen warps of
            // arithmetic, and one would hold the pipeline.  Each TMEM buffer is accumulated by
            // one thread at a time:
            //   thread 0 (warp 16): each own chunk c of pass q into its columns [32 c, Pn) of
            //     buffer X, after the far-field of X (thread 1, pass q - 1) is complete; the A
            //     tiles that later passes read into the cache, and the cached tiles back into
            //     the slots, two items ahead of thread 1;
            //   thread 1 (warp 17): before the last pass, each own chunk into all 256 columns
            //     of pass q + 1 in buffer Y, then its share of the cached chunks 0 .. cb - 1;
            //     one commit on `ydone` per pass marks buffer Y complete.
            const int me = warp - kMmaWarp;
            unsigned char* cache = a.acache + (size_t)blockIdx.x * a.ncache * kStageA;
            const uint32_t cs0 = smem_u32(base + L.cs);
            int64_t G = 0;   // passes so far (all tiles): pass G accumulates in buffer G & 1
            int64_t ny = 0;  // passes so far with a far-field (phases of ydone)
            int64_t cl = 0;  // thread 0: cached tiles loaded
            int64_t cj = 0;  // thread 1: cached tiles consumed
            int s = 0;
            uint32_t ph = 0;
            bool ok = mbar_wait(smem_u32(strip_bar), 0, a.err, 3, a.prof);
            // thread 0: cached chunk `chunk` into the next slot, once thread 1 is done with the
            // slot's previous tile (block: wait for it; otherwise only if it already is)
            auto load = [&](int chunk, bool block) -> int {
                const int slot = (int)(cl % kCSlots);
                const uint32_t ce_bar = smem_u32(cempty + slot), ce_par = (uint32_t)((cl / kCSlots - 1) & 1);
                if (cl >= kCSlots) {
                    if (!block && !mbar_test(ce_bar, ce_par)) return 0;
                    if (block && !mbar_wait(ce_bar, ce_par, a.err, 9, a.prof)) return -1;
                }
                const uint32_t bar = smem_u32(cfull + slot);
                mbar_expect_tx(bar, (uint32_t)kStageA);
                bulk_g2s(cs0 + (uint32_t)(slot * kStageA), cache + (size_t)chunk * kStageA, (uint32_t)kStageA, bar);
                ++cl;
                return 1;
            };
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                for (int q = 0; q < pp.np && ok; ++q, ++G) {
                    const int cb = pp.begin(q), ce = pp.end(q);
                    const int P = kChunk * cb, Pn = kChunk * ce;  // columns: this pass [P, Pn), the next [Pn, Pn + 256)
                    const bool has_y = q + 1 < pp.np;
                    const int k = ce - cb, mC = has_y ? cb : 0;  // own chunks; cached chunks into Y
                    const uint32_t xb = tmem + (uint32_t)((G & 1) * kHalfCols);
                    const uint32_t yb = tmem + (uint32_t)(((G + 1) & 1) * kHalfCols);
                    int u = 0;  // cached chunks of this pass loaded (thread 0) or consumed (thread 1)
                    for (int c = cb; c < ce && ok; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                        const int u_end = (int)((int64_t)mC * (c - cb + 1) / k);  // thread 1's items after chunk c
                        if (me == 0) {
                            if (c == 0 && G >= 2) {
                                // a tile's first pass starts a fresh buffer: pass G - 2 there is read
                                if (!mbar_wait(smem_u32((G & 1) ? tmem_empty1 : tmem_empty),
                                               (uint32_t)(((G - 2) >> 1) & 1), a.err, 4, a.prof)) {
                                    ok = false;
                                    break;
                                }
                            }
                            if (c == cb && q > 0 &&
                                !mbar_wait(smem_u32(ydone), (uint32_t)((ny - 1) & 1), a.err, 13, a.prof)) {
                                // thread 1's far-field of this buffer (pass q - 1) is complete
                                ok = false;
                                break;
                            }
                            if (!mbar_wait(smem_u32(full + s), ph, a.err, 5, a.prof)) {
                                ok = false;
                                break;
                            }
                            tc_fence_after();
                            const uint32_t ahi = smem_u32(base + L.a0 + s * kStageA);
                            mma_chunk_narrow<SK>(xb + (uint32_t)(kChunk * c - P), ahi, strip_hi, strip_lo, 0u,
                                                 Pn - kChunk * c, q == 0 && c == 0);
                            umma_commit(smem_u32(accf + s));
                            umma_commit(smem_u32(empty + s));
                            if (c < a.ncache) {
                                // the chunk's A tile into the cache; the stage may be refilled once
                                // the copy has read it
                                bulk_s2g(cache + (size_t)c * kStageA, ahi, (uint32_t)kStageA);
                                const long long t0 = a.prof ? clock64() : 0;
                                bulk_wait_read0();
                                if (a.prof) atomicAdd(a.prof + 11, (unsigned long long)(clock64() - t0));
                            }
                            mbar_arrive(smem_u32(empty + s));
                            if (mC > 0) {
                                if (c == cb) {
                                    // the cached tiles of chunks < cb are in global memory (the most
                                    // recent store, when there is one, is this chunk's own)
                                    if (c < a.ncache)
                                        bulk_wait_done1();
                                    else
                                        bulk_wait_done0();
                                }
                                // two items ahead of thread 1, as far as the slots are free; the
                                // rest of the pass's items without fail at its last chunk
                                const int want = c + 1 == ce ? mC : (u_end + 2 < mC ? u_end + 2 : mC);
                                while (ok && u < want) {
                                    const int r = load(u, c + 1 == ce);
                                    if (r < 0) ok = false;
                                    if (r <= 0) break;
                                    ++u;
                                }
                            }
                        } else {
                            if (!mbar_wait(smem_u32(full + s), ph, a.err, 5, a.prof)) {
                                ok = false;
                                break;
                            }
                            if (!has_y) {
                                // the last pass has no far-field: the stage's arrival all the same
                                mbar_arrive(smem_u32(empty + s));
                                continue;
                            }
                            if (c == cb && G >= 1) {
                                // Y held pass G - 1: its columns are read
                                if (!mbar_wait(smem_u32(((G + 1) & 1) ? tmem_empty1 : tmem_empty),
                                               (uint32_t)(((G - 1) >> 1) & 1), a.err, 4, a.prof)) {
                                    ok = false;
                                    break;
                                }
                            }
                            tc_fence_after();
                            const uint32_t ahi = smem_u32(base + L.a0 + s * kStageA);
                            mma_chunk_narrow<SK>(yb, ahi, strip_hi, strip_lo, (uint32_t)(Pn - kChunk * c), kHalfCols,
                                                 c == cb);
                            umma_commit(smem_u32(empty + s));
                            for (; u < u_end && ok; ++u, ++cj) {
                                const int slot = (int)(cj % kCSlots);
                                if (!mbar_wait(smem_u32(cfull + slot), (uint32_t)((cj / kCSlots) & 1), a.err, 10,
                                               a.prof)) {
                                    ok = false;
                                    break;
                                }
                                tc_fence_after();
                                mma_chunk_narrow<SK>(yb, cs0 + (uint32_t)(slot * kStageA), strip_hi, strip_lo,
                                                     (uint32_t)(Pn - kChunk * u), kHalfCols, false);
                                umma_commit(smem_u32(cempty + slot));
                            }
                        }
                    }
                    if (has_y) {
                        if (me == 1 && ok) umma_commit(smem_u32(ydone));
                        ++ny;
                    }
                }
            }
            if (me == 0) {
                // after an error: the loads in flight land and the stores finish before the CTA exits;
                // every load issued is of a slot whose fill thread 1 waits for, or the error word is set
                for (int64_t i = cl - kCSlots < 0 ? 0 : cl - kCSlots; i < cl; ++i)
                    mbar_drain(smem_u32(cfull + (int)(i % kCSlots)), (uint32_t)((i / kCSlots) & 1));
                bulk_wait_done0();
            }
        } else if (mbar_wait(smem_u32(strip_bar), 0, a.err, 3, a.prof)) {
            // Pass modes 1 and 2 issue from two threads (warps 16 and 17), thread h the MMAs
            // into TMEM columns [256 h, 256 h + 256) of the pass, so each half is accumulated
            // by one thread; pass mode 0 from one.
            const int me = warp - kMmaWarp;
            int64_t pass = 0;
            int s = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                for (int q = 0; q < pp.np && ok; ++q) {
                    const int cb = pp.begin(q), ce = pp.end(q);
                    for (int c = 0; c < ce; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                        // output columns [lo, hi) of this chunk; TMEM column = output column - toff
                        const bool redraw = PM > 0 && c < cb;
                        const int lo = redraw ? kChunk * cb : kChunk * c, hi = kChunk * ce;
                        const int toff = PM > 0 ? kChunk * cb : 0;
                        const bool first = c == 0;  // first chunk of a pass overwrites
                        if (first) {
                            // the epilogue has read every column of the previous pass
                            if (pass > 0 &&
                                !mbar_wait(smem_u32(tmem_empty), (uint32_t)((pass - 1) & 1), a.err, 4, a.prof)) {
                                ok = false;
                                break;
                            }
                            ++pass;
                            tc_fence_after();
                        }
                        if (!mbar_wait(smem_u32(full + s), ph, a.err, 5, a.prof)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t ahi = smem_u32(base + L.a0 + s * kStageA);
                        const uint32_t alo = ahi + kTileBytes;
                        // B operand: the resident strip, or (pass mode 2, redrawn chunk) the window
                        // in this stage whose row 0 is strip row lo - 32 c
                        const bool win = PM == 2 && redraw;
                        const uint32_t bhi = win ? smem_u32(base + L.f0 + s * FB) : strip_hi;
                        const uint32_t blo = win ? bhi + (uint32_t)WB : strip_lo;
                        const int rbase = win ? lo : kChunk * c;
                        int plo = lo, phi = hi;  // this thread's output columns of the chunk
                        if constexpr (PM > 0) {
                            const int mid = toff + kHalfCols;
                            if (me == 0)
                                phi = phi < mid ? phi : mid;
                            else
                                plo = plo > mid ? plo : mid;
                        }
                        if constexpr (T32) {
                            // TF32: four K = 8 steps per chunk, A in TF32 (SW128) against the
                            // narrow strip's hi and lo halves at row offsets 8 apart
                            for (int col0 = plo; col0 < phi; col0 += 256) {
                                const int n = (phi - col0 < 256) ? (phi - col0) : 256;
                                const uint32_t id = idesc_tf32(n);
                                const uint32_t jrow = (uint32_t)(col0 - rbase);
                                const uint32_t d = tmem + (uint32_t)(col0 - toff);
#pragma unroll
                                for (int ks = 0; ks < kChunk / kStripKT; ++ks) {
                                    const uint64_t da = sdesc_sw128(ahi + 32 * ks);
                                    const uint32_t boff = (jrow + (uint32_t)(kStripKT * (3 - ks))) * 32u;
                                    umma_tf32(d, da, sdesc_sw32(bhi + boff), id, (first && ks == 0) ? 0u : 1u);
                                    umma_tf32(d, da, sdesc_sw32(blo + boff), id, 1u);
                                }
                            }
                        } else {
                            for (int col0 = plo; col0 < phi; col0 += 256) {
                                const int n = (phi - col0 < 256) ? (phi - col0) : 256;
                                const uint32_t id = idesc_f16(n, SK);
                                const uint32_t jrow = (uint32_t)(col0 - rbase);
                                const uint32_t d = tmem + (uint32_t)(col0 - toff);
                                if constexpr (!wide) {
                                    mma_chunk_narrow<SK>(d, ahi, bhi, blo, jrow, n, first);
                                } else {
#pragma unroll
                                for (int ks = 0; ks < 2; ++ks) {
                                    // K half ks: A columns [16 ks, 16 ks + 16); wide strip: row jrow, bytes
                                    // [32 ks, 32 ks + 32); narrow strip: rows from jrow + 16 - 16 ks
                                    const uint64_t dah = sdesc_sw64(ahi + 32 * ks), dal = sdesc_sw64(alo + 32 * ks);
                                    uint64_t dbh, dbl;
                                    if (wide) {
                                        dbh = sdesc_sw64(bhi + jrow * 64 + 32 * ks);
                                        dbl = sdesc_sw64(blo + jrow * 64 + 32 * ks);
                                    } else {
                                        const uint32_t boff = (jrow + (uint32_t)(kStripK * (1 - ks))) * (kStripK * 2);
                                        dbh = sdesc_sw32(bhi + boff);
                                        dbl = sdesc_sw32(blo + boff);
                                    }
                                    umma_f16(d, dah, dbh, id, (first && ks == 0) ? 0u : 1u);
                                    umma_f16(d, dah, dbl, id, 1u);
                                    umma_f16(d, dal, dbh, id, 1u);
                                }
                                }
                            }
                        }
                        umma_commit(smem_u32(empty + s));
                        // the epilogue reads this chunk's columns from one half: its thread signals
                        // them (thread 0 for a redrawn chunk, which the epilogue only counts)
                        if (PM == 0 || me == ((!redraw && kChunk * c - toff >= kHalfCols) ? 1 : 0))
                            umma_commit(smem_u32(accf + s));
                    }
                }
            }
        }
        // drain every issued MMA before TMEM is released
        umma_commit(smem_u32(final_bar));
        mbar_wait(smem_u32(final_bar), 0, a.err, 6);
    }
done:
    if (a.prof && lane == 0) {
        const int role = warp < kProdWarps ? 16 : (warp < kMmaWarp ? 17 : 18);
        atomicAdd(a.prof + role, (unsigned long long)(clock64() - role_t0));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kMmaWarp) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols)
                     : "memory");
    }
    // this CTA's fused payoff sums: one partial row per CTA, merged in fixed order later
    if (a.n_o > 0 && warp >= kEpiWarp0 && warp < kMmaWarp) {
        for (int q = threadIdx.x - kEpiWarp0 * 32; q < a.n_o; q += kEpiWarps * 32) {
            double S1 = 0, C1 = 0, S2 = 0, C2 = 0;
            for (int w = 0; w < kEpiWarps; ++w) {
                const float* os = osum + ((size_t)w * a.n_o + q) * 4;
                neumaier_add(S1, C1, (double)os[0]);
                neumaier_add(S1, C1, -(double)os[1]);
                neumaier_add(S2, C2, (double)os[2]);
                neumaier_add(S2, C2, -(double)os[3]);
            }
            double* pp = a.part + ((size_t)blockIdx.x * a.n_out_total + a.oidx[q]) * 4;
            pp[0] = S1; pp[1] = C1; pp[2] = S2; pp[3] = C2;
        }
    }
}

// --------------------------------------------- job-table (shared) launches
// The serving loop's shared launch: one path kernel over the tiles of many
// requests ("jobs"), each with its own parameters, Philox seed, path range,
// strip and compensator table (a.jobs[j], device memory), its tiles
// [job_tile0[j], job_tile0[j + 1]) of the launch.  One TMEM pass (N <= 512),
// the RT estimator, Philox normals, (Ivdt, IsvdW) per path out; payoffs in
// the job-table payoff kernel.  Each CTA takes a contiguous range of tiles,
// so it meets a new job rarely: then the MMA issuer reloads the strip once
// every MMA issued on the old one has completed, and the epilogue warps the
// compensator table after the barrier that ended the last tile.  The
// launch's own arguments give the shared-memory layout (largest Np and group
// count of its jobs), the error word and the TMEM allocation.
// Per path it performs k_mixed_gemm's operations in the same order, so a
// request's results are the same alone and in any mix.  It is a kernel of
// its own, not a template flag of k_mixed_gemm: the per-tile job lookup
// folded into that kernel made its ordinary launches 10% slower (measured).
template <int SK>
__global__ void __launch_bounds__(kThreads, 1) k_mixed_gemm_jobs(const __grid_constant__ MixedArgs a)
{
    constexpr int NS = 2;
    constexpr int kStageFB = stage_f_bytes(NS);
    constexpr bool T32 = SK == 2;
    extern __shared__ unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const SmemLayout L = smem_layout(a.Np, a.stages, a.n_g, 0, NS, T32);
    unsigned char* strip = base + L.strip;
    float* acc_s = (float*)(base + L.acc);
    float* beta_s = (float*)(base + L.beta);
    uint64_t* bars = (uint64_t*)(base + L.bars);
    const int S = a.stages;
    uint64_t* full = bars;       // [S]
    uint64_t* empty = bars + 3;  // [S]
    uint64_t* accf = bars + 6;   // [S]
    uint64_t* tmem_empty = bars + 9;
    uint64_t* strip_bar = bars + 10;
    uint64_t* final_bar = bars + 11;
    uint32_t* tmem_holder = (uint32_t*)(bars + 12);
    uint64_t* strip_free = bars + 13;  // every MMA issued on the old strip has completed
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // this CTA's tiles [t_first, t_last), starting in job jb
    const int64_t T = a.job_tile0[a.n_jobs];
    const int64_t t_first = T * blockIdx.x / gridDim.x, t_last = T * (blockIdx.x + 1) / gridDim.x;
    int jb = 0;
    while (jb + 1 < a.n_jobs && t_first >= a.job_tile0[jb + 1]) ++jb;
    const MixedArgs& J0 = a.jobs[jb];
    auto strip_bytes_of = [](int Np) { return (uint32_t)(T32 ? strip_smem_bytes_t32(Np) : strip_smem_bytes(Np)); };

    if (threadIdx.x == kMmaWarp * 32) {
        for (int s = 0; s < S; ++s) {
            mbar_init(smem_u32(full + s), kProdWarps);
            mbar_init(smem_u32(empty + s), 1 + kEpiWarps);
            mbar_init(smem_u32(accf + s), 1);
        }
        mbar_init(smem_u32(tmem_empty), kEpiWarps);
        mbar_init(smem_u32(strip_bar), 1);
        mbar_init(smem_u32(final_bar), 1);
        mbar_init(smem_u32(strip_free), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const uint32_t nb = strip_bytes_of(J0.Np);
        mbar_expect_tx(smem_u32(strip_bar), nb);
        bulk_g2s(smem_u32(strip), J0.strip, nb, smem_u32(strip_bar));
    }
    if (warp == kMmaWarp) {
        __syncwarp();
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int i = threadIdx.x; i < J0.n_g * J0.Np; i += blockDim.x) beta_s[i] = J0.beta[i];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    if (warp < kProdWarps) {
        // ------------------------------------------------------- producers
        const int p = threadIdx.x & (kTileM - 1);
        const int h = threadIdx.x >> 7;
        PhiloxKeys keys = philox_keys(J0.seed);
        int s = 0, j = jb;
        uint32_t ph = 0;
        for (int64_t it = t_first; it < t_last; ++it) {
            const int jp = j;
            while (it >= a.job_tile0[j + 1]) ++j;
            if (j != jp) keys = philox_keys(a.jobs[j].seed);
            const MixedArgs& J = a.jobs[j];
            const int64_t m = (it - a.job_tile0[j]) * kTileM + p;
            const bool valid = m < J.B;
            const uint64_t gpath = (uint64_t)(J.path0 + m);
            for (int c = 0; c < J.nc; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                if (!mbar_wait_warp(smem_u32(empty + s), ph ^ 1u, a.err, 1)) goto done;
                unsigned char* st = base + L.a0 + s * kStageA;
                float* w1s = (float*)(base + L.f0 + s * kStageFB);
                produce_chunk<SK, false, false>(J, keys, gpath, valid, m, p, h, c, false, st, w1s);
                fence_proxy_async();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(full + s));
            }
        }
    } else if (warp < kMmaWarp) {
        // -------------------------------------------------------- epilogue
        const int ew = warp - kEpiWarp0;
        const int wg = ew >> 2;
        const int quad = warp & 3;
        const int p = quad * 32 + lane;
        const uint32_t tlane = tmem + ((uint32_t)(quad * 32) << 16);
        float* my_acc = acc_s + (size_t)wg * a.n_g * NS * kTileM;
        float* w10_s = acc_s + (size_t)2 * a.n_g * NS * kTileM;
        int s = 0, j = jb;
        uint32_t ph = 0;
        for (int64_t it = t_first; it < t_last; ++it) {
            const int jp = j;
            while (it >= a.job_tile0[j + 1]) ++j;
            const MixedArgs& J = a.jobs[j];
            if (j != jp) {
                // every epilogue warp finished the last tile at the barrier that ended it
                for (int i = threadIdx.x - kEpiWarp0 * 32; i < J.n_g * J.Np; i += kEpiWarps * 32) beta_s[i] = J.beta[i];
                asm volatile("bar.sync 1, %0;" ::"r"(kEpiWarps * 32) : "memory");
            }
            const int Np = J.Np, nc = J.nc;
            const int64_t m = (it - a.job_tile0[j]) * kTileM + p;
            const bool valid = m < J.B;
            for (int g = 0; g < J.n_g; ++g)
#pragma unroll
                for (int t = 0; t < NS; ++t) my_acc[(NS * g + t) * kTileM + p] = 0.f;
            for (int c = 0; c < nc; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                if (!mbar_wait_warp(smem_u32(full + s), ph, a.err, 7)) goto done;
                const bool pass_end = c == nc - 1;
                const bool has_next = c + 1 < nc;
                const int sn = (s + 1 == S) ? 0 : s + 1;
                if ((kEpiWGs == 1 || wg == 1) && has_next &&
                    !mbar_wait_warp(smem_u32(full + sn), sn == 0 ? ph ^ 1u : ph, a.err, 8))
                    goto done;
                if (!mbar_wait_warp(smem_u32(accf + s), ph, a.err, 2)) goto done;
                tc_fence_after();
                const float* w1s = (const float*)(base + L.f0 + s * kStageFB);
                const float* w1ps = w1s + kFW1p;
#pragma unroll 1
                for (int hh = wg; hh < 2; hh += kEpiWGs) {
                    const int j0 = 16 * hh;
                    float w1v[16], w1pv[16];
#pragma unroll
                    for (int jj = 0; jj < 16; jj += 4) {
                        const int at = ftile_at(p, j0 + jj);
                        const float4 u = *(const float4*)(w1s + at), v = *(const float4*)(w1ps + at);
                        w1v[jj] = u.x; w1v[jj + 1] = u.y; w1v[jj + 2] = u.z; w1v[jj + 3] = u.w;
                        w1pv[jj] = v.x; w1pv[jj + 1] = v.y; w1pv[jj + 2] = v.z; w1pv[jj + 3] = v.w;
                    }
                    const float* nexts = (const float*)(base + L.f0 + sn * kStageFB);
                    const float w_after = (hh == 0) ? w1s[ftile_at(p, 16)] : (!has_next ? 0.f : nexts[ftile_at(p, 0)]);
                    float x[16];
                    tmem_ld16(tlane + (uint32_t)(kChunk * c + j0), x);
                    if (pass_end && hh + kEpiWGs >= 2) {
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(smem_u32(tmem_empty));
                    }
                    float wn[16];
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj) {
                        const float w1 = w1v[jj];
                        x[jj] = x[jj] + J.a1 * w1 + J.a2 * w1pv[jj];
                        if (jj > 0) wn[jj - 1] = w1;
                        if (jj == 0 && j0 == 0 && c == 0) w10_s[p] = w1;
                    }
                    wn[15] = w_after;
                    for (int g = 0; g < J.n_g; ++g) {
                        const float ah = J.alpha[g];
                        const float* btp = beta_s + g * Np + kChunk * c + j0;
                        float bt[16];
#pragma unroll
                        for (int jj = 0; jj < 16; jj += 4) {
                            const float4 u = *(const float4*)(btp + jj);
                            bt[jj] = u.x; bt[jj + 1] = u.y; bt[jj + 2] = u.z; bt[jj + 3] = u.w;
                        }
                        const int lim = J.nsteps[g] - 1 - kChunk * c - j0;
                        float sv = 0.f, swv = 0.f;
                        if (lim >= 16) {
#pragma unroll
                            for (int jj = 0; jj < 16; ++jj) {
                                const float su = ex2_approx(fmaf(ah, x[jj], -bt[jj]));
                                sv = fmaf(su, su, sv);
                                swv = fmaf(su, wn[jj], swv);
                            }
                        } else {
#pragma unroll
                            for (int jj = 0; jj < 16; ++jj) {
                                if (jj < lim) {
                                    const float su = ex2_approx(fmaf(ah, x[jj], -bt[jj]));
                                    sv = fmaf(su, su, sv);
                                    swv = fmaf(su, wn[jj], swv);
                                }
                            }
                        }
                        my_acc[(NS * g) * kTileM + p] += sv;
                        my_acc[(NS * g + 1) * kTileM + p] += swv;
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(empty + s));
            }
            asm volatile("bar.sync 1, %0;" ::"r"(kEpiWarps * 32) : "memory");
            if (wg == 0 && valid) {
                const float w1_0 = w10_s[p];
                for (int g = 0; g < J.n_g; ++g) {
                    float sv = acc_s[(NS * g) * kTileM + p], sw2 = acc_s[(NS * g + 1) * kTileM + p];
                    if (kEpiWGs == 2) {
                        sv += acc_s[((size_t)a.n_g * NS + NS * g) * kTileM + p];
                        sw2 += acc_s[((size_t)a.n_g * NS + NS * g + 1) * kTileM + p];
                    }
                    J.ivb[(size_t)(J.g0 + g) * J.B + m] =
                        make_float2(J.dt[g] * (J.xi + sv), J.sdt[g] * fmaf(J.sqrt_xi, w1_0, sw2));
                }
            }
            asm volatile("bar.sync 1, %0;" ::"r"(kEpiWarps * 32) : "memory");
        }
    } else if (lane == 0) {
        // ------------------------------------------------------ MMA issuer
        const uint32_t strip_hi = smem_u32(strip);
        uint32_t strip_lo = strip_hi + strip_bytes_of(J0.Np) / 2;
        if (mbar_wait(smem_u32(strip_bar), 0, a.err, 3)) {
            int64_t pass = 0;
            int s = 0, j = jb;
            uint32_t ph = 0, strip_loads = 1, strip_frees = 0;
            bool ok = true;
            for (int64_t it = t_first; it < t_last && ok; ++it) {
                const int jp = j;
                while (it >= a.job_tile0[j + 1]) ++j;
                const MixedArgs& J = a.jobs[j];
                if (j != jp) {
                    // the new job's strip, once every MMA issued on the old one has completed
                    umma_commit(smem_u32(strip_free));
                    if (!mbar_wait(smem_u32(strip_free), strip_frees & 1u, a.err, 9)) break;
                    ++strip_frees;
                    const uint32_t nb = strip_bytes_of(J.Np);
                    mbar_expect_tx(smem_u32(strip_bar), nb);
                    bulk_g2s(strip_hi, J.strip, nb, smem_u32(strip_bar));
                    if (!mbar_wait(smem_u32(strip_bar), strip_loads & 1u, a.err, 3)) break;
                    ++strip_loads;
                    strip_lo = strip_hi + nb / 2;
                }
                const int hi = kChunk * J.nc;
                for (int c = 0; c < J.nc; ++c, s = (s + 1 == S) ? 0 : s + 1, ph ^= (s == 0)) {
                    const bool first = c == 0;
                    if (first) {
                        if (pass > 0 &&
                            !mbar_wait(smem_u32(tmem_empty), (uint32_t)((pass - 1) & 1), a.err, 4)) {
                            ok = false;
                            break;
                        }
                        ++pass;
                        tc_fence_after();
                    }
                    if (!mbar_wait(smem_u32(full + s), ph, a.err, 5)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t ahi = smem_u32(base + L.a0 + s * kStageA);
                    const uint32_t alo = ahi + kTileBytes;
                    for (int col0 = kChunk * c; col0 < hi; col0 += 256) {
                        const int n = (hi - col0 < 256) ? (hi - col0) : 256;
                        const uint32_t jrow = (uint32_t)(col0 - kChunk * c);
                        const uint32_t d = tmem + (uint32_t)col0;
                        if constexpr (T32) {
                            const uint32_t id = idesc_tf32(n);
#pragma unroll
                            for (int ks = 0; ks < kChunk / kStripKT; ++ks) {
                                const uint64_t da = sdesc_sw128(ahi + 32 * ks);
                                const uint32_t boff = (jrow + (uint32_t)(kStripKT * (3 - ks))) * 32u;
                                umma_tf32(d, da, sdesc_sw32(strip_hi + boff), id, (first && ks == 0) ? 0u : 1u);
                                umma_tf32(d, da, sdesc_sw32(strip_lo + boff), id, 1u);
                            }
                        } else {
                            const uint32_t id = idesc_f16(n, SK);
#pragma unroll
                            for (int ks = 0; ks < 2; ++ks) {
                                const uint64_t dah = sdesc_sw64(ahi + 32 * ks), dal = sdesc_sw64(alo + 32 * ks);
                                const uint64_t dbh = sdesc_sw64(strip_hi + jrow * 64 + 32 * ks);
                                const uint64_t dbl = sdesc_sw64(strip_lo + jrow * 64 + 32 * ks);
                                umma_f16(d, dah, dbh, id, (first && ks == 0) ? 0u : 1u);
                                umma_f16(d, dah, dbl, id, 1u);
                                umma_f16(d, dal, dbh, id, 1u);
                            }
                        }
                    }
                    umma_commit(smem_u32(empty + s));
                    umma_commit(smem_u32(accf + s));
                }
            }
        }
        umma_commit(smem_u32(final_bar));
        mbar_wait(smem_u32(final_bar), 0, a.err, 6);
    }
done:
    tc_fence_before();
    __syncthreads();
    if (warp == kMmaWarp) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols)
                     : "memory");
    }
}

// ----------------------------------------------- FP32 payoffs, FP64 sums
constexpr int kOPB32 = 8;

// Plain Monte Carlo payoff in FP32: S_T = exp(rho IsvdW + sqrt(1 - rho^2) IsvdWp
// - Ivdt / 2) (the FP64 form's mc_payoff), payoff max(S_T - K, 0).
__device__ __forceinline__ float mc_payoff_f32(float Ivdt, float IsvdW, float IsvdWp, float rho, float K)
{
    const float lnS = fmaf(rho, IsvdW, fmaf(sqrtf(fmaxf(1.0f - rho * rho, 0.0f)), IsvdWp, -0.5f * Ivdt));
    return fmaxf(ex2_approx(1.4426950408889634f * lnS) - K, 0.0f);
}

// One block of the FP32 payoff sums: chunk c (paths [256 G c, 256 G (c + 1)))
// and outputs [o0, o0 + 8).  Shared by the per-request and job-table kernels,
// so a request's sums do not depend on which of them ran.
template <bool MC>
__device__ __forceinline__ void payoff_sums_block(const OutDev* __restrict__ outs, int n_out,
                                                  const float2* __restrict__ ivb, int64_t B, int G,
                                                  double* __restrict__ part, const float* __restrict__ ivq, int c,
                                                  int o0, double (*red)[kOPB32][2])
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float rho[kOPB32], K[kOPB32], lnK[kOPB32];
    int vg[kOPB32];
#pragma unroll
    for (int q = 0; q < kOPB32; ++q) {
        const int i = o0 + q;
        const OutDev od = (i < n_out) ? outs[i] : OutDev{0.0, 1.0, -1, 0};
        rho[q] = (float)od.rho; K[q] = (float)od.K; lnK[q] = logf((float)od.K); vg[q] = od.vg;
    }
    // each thread sums its own G paths in FP32 (G <= a few dozen), FP64 from the warp level up
    float s1[kOPB32], s2[kOPB32];
#pragma unroll
    for (int q = 0; q < kOPB32; ++q) { s1[q] = 0.f; s2[q] = 0.f; }
    for (int sub = 0; sub < G; ++sub) {
        const int64_t m = ((int64_t)c * G + sub) * 256 + threadIdx.x;
        if (m >= B) break;
        int cur = -1;
        float2 iv = make_float2(0.f, 0.f);
        float ip = 0.f, srho = 0.f;
        RtSpot sp{};
#pragma unroll
        for (int q = 0; q < kOPB32; ++q) {
            if (vg[q] < 0) continue;
            bool fresh = false;
            if (vg[q] != cur) {
                cur = vg[q];
                iv = ivb[(size_t)cur * B + m];
                if (MC) ip = ivq[(size_t)cur * B + m];
                fresh = true;
            }
            // the strike-independent terms once per (group, rho): outputs of one
            // ParamTot tuple share them
            if (!MC && (fresh || rho[q] != srho)) {
                sp = rt_spot_f32(iv.x, iv.y, rho[q]);
                srho = rho[q];
            }
            const float x = MC ? mc_payoff_f32(iv.x, iv.y, ip, rho[q], K[q]) : rt_payoff_f32(sp, K[q], lnK[q]);
            s1[q] += x;
            s2[q] = fmaf(x, x, s2[q]);
        }
    }
    // warp tree in FP32 (GB300's FP64 pipe is far too slow for warp-wide
    // shuffles), one FP64 value per warp and output
#pragma unroll
    for (int q = 0; q < kOPB32; ++q) {
        float a = s1[q], b = s2[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0) { red[w][q][0] = (double)a; red[w][q][1] = (double)b; }
    }
    __syncthreads();
    if (threadIdx.x < kOPB32 && o0 + (int)threadIdx.x < n_out) {
        const int q = threadIdx.x;
        double S = 0, CS = 0, S2 = 0, CS2 = 0;
        for (int k = 0; k < 8; ++k) {
            neumaier_add(S, CS, red[k][q][0]);
            neumaier_add(S2, CS2, red[k][q][1]);
        }
        double* pp = part + ((size_t)c * n_out + o0 + q) * 4;
        pp[0] = S; pp[1] = CS; pp[2] = S2; pp[3] = CS2;
    }
}

template <bool MC>
__global__ void __launch_bounds__(256) k_payoff_sums_f32(const OutDev* __restrict__ outs, int n_out,
                                                         const float2* __restrict__ ivb, int64_t B, int G,
                                                         double* __restrict__ part, const float* __restrict__ ivq)
{
    __shared__ double red[8][kOPB32][2];
    payoff_sums_block<MC>(outs, n_out, ivb, B, G, part, ivq, blockIdx.x, blockIdx.y * kOPB32, red);
}

// Job-table form: block b of the launch is block b - jobs[k].block0 of job k
// (chunk-major as in the per-request grid: chunk = local % nchunks, output
// block = local / nchunks).
__global__ void __launch_bounds__(256) k_payoff_sums_f32_jobs(const PayoffJob* __restrict__ jobs, int n_jobs)
{
    __shared__ double red[8][kOPB32][2];
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {  // last job whose first block is <= blockIdx.x
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].block0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const PayoffJob& J = jobs[lo];
    const int local = (int)((int64_t)blockIdx.x - J.block0);
    payoff_sums_block<false>(J.outs, J.n_out, J.ivb, J.B, J.G, J.part, nullptr, local % J.nchunks,
                             (local / J.nchunks) * kOPB32, red);
}

void launch_payoff_sums_f32(const OutDev* outs, int n_out, const void* ivb, int64_t B, int G, double* part,
                            int nchunks, cudaStream_t st, const float* ivq)
{
    dim3 grid(nchunks, (n_out + kOPB32 - 1) / kOPB32);
    if (ivq) k_payoff_sums_f32<true><<<grid, 256, 0, st>>>(outs, n_out, (const float2*)ivb, B, G, part, ivq);
    else k_payoff_sums_f32<false><<<grid, 256, 0, st>>>(outs, n_out, (const float2*)ivb, B, G, part, ivq);
    count_launch();
}

void launch_payoff_sums_f32_jobs(const PayoffJob* jobs, int n_jobs, int64_t blocks, cudaStream_t st)
{
    k_payoff_sums_f32_jobs<<<(unsigned)blocks, 256, 0, st>>>(jobs, n_jobs);
    count_launch();
}

// Per-path payoffs in FP32 (the mixed form of the quadrature entry points):
// payoff[m * n_out + i] for paths m < B, as double.
template <bool MC>
__global__ void k_payoff_store_f32(const OutDev* __restrict__ outs, int n_out, const float2* __restrict__ ivb,
                                   const float* __restrict__ ivq, int64_t B, double* __restrict__ payoff)
{
    const int64_t total = B * n_out;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = idx / n_out;
        const int i = (int)(idx - m * n_out);
        const OutDev od = outs[i];
        const size_t at = (size_t)od.vg * B + m;
        const float2 iv = ivb[at];
        const float rho = (float)od.rho, K = (float)od.K;
        payoff[idx] = MC ? (double)mc_payoff_f32(iv.x, iv.y, ivq[at], rho, K)
                         : (double)rt_payoff_f32(rt_spot_f32(iv.x, iv.y, rho), K, logf(K));
    }
}

void launch_payoff_store_f32(const OutDev* outs, int n_out, const void* ivb, const float* ivq, int64_t B,
                             double* payoff, cudaStream_t st)
{
    const int64_t total = B * n_out;
    int64_t blocks = (total + 255) / 256;
    if (blocks > (1 << 20)) blocks = 1 << 20;
    if (ivq)
        k_payoff_store_f32<true><<<(unsigned)blocks, 256, 0, st>>>(outs, n_out, (const float2*)ivb, ivq, B, payoff);
    else
        k_payoff_store_f32<false><<<(unsigned)blocks, 256, 0, st>>>(outs, n_out, (const float2*)ivb, ivq, B, payoff);
    count_launch();
}

// ------------------------------------------- control variate, FP32 payoffs
// The Romano-Touzi estimator with the McCrickerd-Pakkanen control variate on
// antithetic paths (ML_console_ST/RBergomi.cpp:218-306), priced from the
// mixed path kernel's FP32 sums: f = X + alpha Y with X = BS(spot, K,
// sqrt((1 - rho^2) Ivdt)) and Y = BS(spot, K, sqrt(rho^2 (Q - Ivdt))) -- Q_max
// in place of Q where Q <= Ivdt, counted -- averaged over W and -W.
__device__ __forceinline__ float cv_half_f32(float Ivdt, float IsvdW, float rho, float K, float lnK, float alpha,
                                             float Q, float Qmax, unsigned& exc)
{
    const RtSpot r = rt_spot_f32(Ivdt, IsvdW, rho);
    const float x = rt_payoff_f32(r, K, lnK);
    const bool inside = Q > Ivdt;
    if (!inside) ++exc;
    RtSpot ry = r;
    const float v2 = rho * rho * ((inside ? Q : Qmax) - Ivdt);
    ry.deg = !(v2 > 0.0f);
    ry.rv = rsqrt_approx(v2);
    ry.vol = v2 * ry.rv;
    return fmaf(alpha, rt_payoff_f32(ry, K, lnK), x);
}

// One block per (chunk c of 256 G paths, 8 outputs), as k_payoff_sums_f32.
// The path kernel ran twice with xi = 0 in its final sums: ivb with the
// variance exponent's coefficient as is, ivn with it negated, which is the
// antithetic path -W exactly (X is linear in the normals, so X(-W) = -X(W)).
// Per group g and path: Ivdt = raw.x + dt xi_g; IsvdW = raw.y + sdt sqrt(xi_g)
// W1_0 for W and -(raw.y + sdt sqrt(xi_g) W1_0) for -W, W1_0 redrawn from the
// path's Philox stream (the path kernel's first W1).
__global__ void __launch_bounds__(256) k_payoff_sums_cv_f32(const OutDev* __restrict__ outs,
                                                            const VGDev* __restrict__ vgs, int n_out,
                                                            const float2* __restrict__ ivb,
                                                            const float2* __restrict__ ivn, int64_t B, int G,
                                                            uint64_t seed, int64_t path0,
                                                            const double* __restrict__ alpha,
                                                            const double* __restrict__ Q, float Qmax,
                                                            double* __restrict__ part,
                                                            unsigned long long* __restrict__ count)
{
    __shared__ double red[8][kOPB32][2];
    const int c = blockIdx.x, o0 = blockIdx.y * kOPB32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float rho[kOPB32], K[kOPB32], lnK[kOPB32], al[kOPB32], qq[kOPB32];
    int vg[kOPB32];
    unsigned exc[kOPB32];
#pragma unroll
    for (int q = 0; q < kOPB32; ++q) {
        const int i = o0 + q;
        const OutDev od = (i < n_out) ? outs[i] : OutDev{0.0, 1.0, -1, 0};
        rho[q] = (float)od.rho; K[q] = (float)od.K; lnK[q] = logf((float)od.K); vg[q] = od.vg;
        al[q] = (i < n_out) ? (float)alpha[i] : 0.f;
        qq[q] = (i < n_out) ? (float)Q[i] : 0.f;
        exc[q] = 0;
    }
    const PhiloxKeys keys = philox_keys(seed);
    float s1[kOPB32], s2[kOPB32];
#pragma unroll
    for (int q = 0; q < kOPB32; ++q) { s1[q] = 0.f; s2[q] = 0.f; }
    for (int sub = 0; sub < G; ++sub) {
        const int64_t m = ((int64_t)c * G + sub) * 256 + threadIdx.x;
        if (m >= B) break;
        const uint4 x0 = philox_group(keys, (uint64_t)(path0 + m), 0u, 0u);
        float w10, w11;
        box_muller_f32(x0.x, x0.y, w10, w11);
        int cur = -1;
        float ipx = 0.f, ipy = 0.f, inx = 0.f, iny = 0.f;
#pragma unroll
        for (int q = 0; q < kOPB32; ++q) {
            if (vg[q] < 0) continue;
            if (vg[q] != cur) {
                cur = vg[q];
                const VGDev gd = vgs[cur];
                const float dtxi = (float)(gd.dt * gd.xi), c0 = (float)(gd.sdt * sqrt(gd.xi)) * w10;
                const float2 rp = ivb[(size_t)cur * B + m], rn = ivn[(size_t)cur * B + m];
                ipx = rp.x + dtxi;
                ipy = rp.y + c0;
                inx = rn.x + dtxi;
                iny = -(rn.y + c0);
            }
            const float x = 0.5f * (cv_half_f32(ipx, ipy, rho[q], K[q], lnK[q], al[q], qq[q], Qmax, exc[q]) +
                                    cv_half_f32(inx, iny, rho[q], K[q], lnK[q], al[q], qq[q], Qmax, exc[q]));
            s1[q] += x;
            s2[q] = fmaf(x, x, s2[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < kOPB32; ++q) {
        float a = s1[q], b = s2[q];
        unsigned e = exc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            e += __shfl_xor_sync(0xffffffffu, e, o);
        }
        if (lane == 0) {
            red[w][q][0] = (double)a;
            red[w][q][1] = (double)b;
            if (e && o0 + q < n_out) atomicAdd(count + o0 + q, (unsigned long long)e);
        }
    }
    __syncthreads();
    if (threadIdx.x < kOPB32 && o0 + (int)threadIdx.x < n_out) {
        const int q = threadIdx.x;
        double S = 0, CS = 0, S2 = 0, CS2 = 0;
        for (int k = 0; k < 8; ++k) {
            neumaier_add(S, CS, red[k][q][0]);
            neumaier_add(S2, CS2, red[k][q][1]);
        }
        double* pp = part + ((size_t)c * n_out + o0 + q) * 4;
        pp[0] = S; pp[1] = CS; pp[2] = S2; pp[3] = CS2;
    }
}

void launch_payoff_sums_cv_f32(const OutDev* outs, const VGDev* vgs, int n_out, const void* ivb, const void* ivn,
                               int64_t B, int G, uint64_t seed, int64_t path0, const double* alpha, const double* Q,
                               double Qmax, double* part, unsigned long long* count, int nchunks, cudaStream_t st)
{
    const dim3 grid((unsigned)nchunks, (unsigned)((n_out + kOPB32 - 1) / kOPB32));
    k_payoff_sums_cv_f32<<<grid, 256, 0, st>>>(outs, vgs, n_out, (const float2*)ivb, (const float2*)ivn, B, G, seed,
                                                path0, alpha, Q, (float)Qmax, part, count);
    count_launch();
}

// Failure-detection check: one warp waits, through the pricing kernels'
// bounded-wait helper, on an mbarrier that nothing arrives on, with a 20 ms
// limit; the expiry records `site` in the error word, as a pipeline wait
// would, and the kernel returns.
constexpr uint64_t kProbeWaitNs = 20000000ull;
__global__ void k_wait_probe(unsigned int* err, unsigned int site)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(smem_u32(&bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();
    const bool ok = mbar_wait<kProbeWaitNs>(smem_u32(&bar), 0, err, site);
    if (__all_sync(0xffffffffu, ok) && threadIdx.x == 0) atomicExch(err, 0xffffffffu);  // cannot happen: nothing arrives
}

int launch_wait_probe(unsigned int* err, unsigned int site, cudaStream_t st)
{
    k_wait_probe<<<1, 32, 0, st>>>(err, site);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ------------------------------------------------------------------- host
namespace {

uint16_t to_bf16(float f)
{
    __nv_bfloat16 h = __float2bfloat16_rn(f);
    uint16_t u;
    std::memcpy(&u, &h, 2);
    return u;
}
float from_bf16(uint16_t u)
{
    __nv_bfloat16 h;
    std::memcpy(&h, &u, 2);
    return __bfloat162float(h);
}
uint16_t to_f16(float f)
{
    __half h = __float2half_rn(f);
    uint16_t u;
    std::memcpy(&u, &h, 2);
    return u;
}
float from_f16(uint16_t u)
{
    __half h;
    std::memcpy(&h, &u, 2);
    return __half2float(h);
}

// The strip image the MMA descriptors expect, hi/lo 16-bit halves:
//   wide   S[j][k] = Gamma[j - k], rows j in [0, Np), SW64 K-major: row j at
//          j * 64 bytes, 16-byte chunk (k / 8) XOR ((j / 2) mod 4);
//   narrow P[r][k] = Gamma[r - 16 - k], rows r in [0, Np + 16), SW32 K-major:
//          row r at r * 32 bytes, 16-byte chunk (k / 8) XOR ((r / 4) mod 2);
// zero where the Gamma index is negative or >= N.
// The near-field term a1 W1_j stays out of the split products: the epilogue
// adds it from the FP32 normal, which keeps X an order of magnitude closer
// to FP64 than folding a1 into the strip's diagonal (measured; no speed-up).
// FP32 -> TF32 (10-bit mantissa) rounded to nearest even, as the FP32 bit
// pattern with the low 13 bits zero.
float to_tf32(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0xFFFu + ((u >> 13) & 1u);
    u &= ~0x1FFFu;
    std::memcpy(&f, &u, 4);
    return f;
}

// sk: split kind, 0 FP16 / 1 BF16 halves (wide or narrow 16-bit strip) or
// 2 TF32 halves (the narrow TF32 strip, P[r][k] = Gamma[r - 24 - k], 8 FP32 per
// 32-byte SW32 row).
void build_strip(const double* gamma, int N, int Np, int sk, unsigned char* img)
{
    // Row r of every strip form holds Gamma[r - lead - k] for k = 0 .. kw - 1,
    // in 16-byte chunks of consecutive k permuted by the row's swizzle.  Along
    // a chunk the Gamma index falls by one per element, so each chunk is a
    // 16-byte run of the hi / lo values in reversed order: the N distinct
    // values are split once and every chunk is one copy (the element-wise
    // build took ~100 us at N = 512, as much as the rest of a call's planning).
    const int esz = (sk == 2) ? 4 : 2;                        // bytes per element
    const bool wide = sk != 2 && strip_k(Np) == kChunk;
    const int kw = (sk == 2) ? kStripKT : (wide ? kChunk : kStripK);
    const int lead = (sk == 2) ? kLeadT : (wide ? 0 : kStripK);
    const int rows = wide ? Np : Np + lead;
    const int per = 16 / esz;                                 // elements per chunk
    const size_t half = (size_t)rows * kw * esz;
    // reversed, zero-padded: rev[pad + i] holds Gamma[N - 1 - i] (i in [0, N))
    const int pad = kw + lead + 32;
    std::vector<unsigned char> rh((size_t)(N + 2 * pad) * esz, 0), rl((size_t)(N + 2 * pad) * esz, 0);
    for (int d = 0; d < N; ++d) {
        const size_t at = (size_t)(pad + N - 1 - d) * esz;
        if (sk == 2) {
            const float hi = to_tf32((float)gamma[d]);
            const float lo = to_tf32((float)(gamma[d] - (double)hi));
            std::memcpy(&rh[at], &hi, 4);
            std::memcpy(&rl[at], &lo, 4);
        } else {
            const uint16_t hi = sk ? to_bf16((float)gamma[d]) : to_f16((float)gamma[d]);
            const uint16_t lo = sk ? to_bf16((float)(gamma[d] - (double)from_bf16(hi)))
                                   : to_f16((float)(gamma[d] - (double)from_f16(hi)));
            std::memcpy(&rh[at], &hi, 2);
            std::memcpy(&rl[at], &lo, 2);
        }
    }
    std::memset(img, 0, 2 * half);
    for (int r = 0; r < rows; ++r) {
        // the swizzle of row r: SW64 (wide) XORs the chunk with (r / 2) mod 4, SW32 with (r / 4) mod 2
        const int sw = wide ? ((r >> 1) & 3) : ((r >> 2) & 1);
        for (int c = 0; c < kw / per; ++c) {
            // chunk c covers k = per c .. per c + per - 1: Gamma indices r - lead - per c down by one
            const int i0 = N - 1 - (r - lead - per * c);  // rev index of its first element
            const size_t src = (size_t)(pad + i0) * esz, dst = (size_t)r * kw * esz + (size_t)((c ^ sw) * 16);
            std::memcpy(img + dst, &rh[src], 16);
            std::memcpy(img + half + dst, &rl[src], 16);
        }
    }
}

}  // namespace

// Attributes of the current device the planner needs, queried once per
// device ordinal (cudaGetDeviceProperties costs far more than the rest of a
// request's planning, and the serving loop plans every request).
struct DevInfo {
    int major, sms, optin;
};
static bool device_info(DevInfo* out)
{
    static std::mutex mu;
    static std::map<int, DevInfo> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it == cache.end()) {
        DevInfo d{};
        if (cudaDeviceGetAttribute(&d.major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&d.optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        it = cache.emplace(dev, d).first;
    }
    *out = it->second;
    return true;
}

void mixed_table_range(const MixedJob& job, int i, size_t* off, size_t* bytes)
{
    const MixedLaunch& r = job.launches[i];
    if (job.backend == RBG_CONV_GEMM) {
        *off = r.off_strip;
        *bytes = (size_t)strip_bytes_sk(r.args.Np, job.split == RBG_SPLIT_TF32X2);
    } else {
        *off = r.off_spec;
        *bytes = (size_t)r.args.L * 8;
    }
}

void mixed_twiddle_range(const MixedJob& job, size_t* off, size_t* bytes)
{
    *off = job.off_tw;
    *bytes = (job.backend == RBG_CONV_FFT && !job.launches.empty()) ? (size_t)job.launches[0].args.L * 8 : 0;
}

// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum, once per (device, kernel): every launch then takes any size the
// planner accepted, with no attribute call on the launch path.
static cudaError_t allow_max_smem(void (*kern)(MixedArgs))
{
    static std::mutex mu;
    static std::set<std::pair<int, uintptr_t>> done;  // (device, kernel address)
    DevInfo dv;
    int dev = 0;
    if (!device_info(&dv) || cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return cudaErrorInvalidDevice;
    }
    std::lock_guard<std::mutex> lk(mu);
    const std::pair<int, uintptr_t> key{dev, reinterpret_cast<uintptr_t>(kern)};
    if (done.count(key)) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dv.optin);
    if (e == cudaSuccess) done.insert(key);
    return e;
}

int mixed_prepare(const Plan& plan, const rbg_options& o, int64_t M, MixedJob& job, std::string& err,
                  int64_t max_batch, bool mc, bool tile_cache)
{
    DevInfo dv;
    if (!device_info(&dv)) {
        err = "device attribute query failed";
        return RBG_ERR_CUDA;
    }
    if (dv.major != 10) {
        err = "mixed form needs a Blackwell (sm_10x) GPU with tcgen05";
        return RBG_ERR_UNSUPPORTED;
    }
    if (o.conv == RBG_CONV_DIRECT) {
        err = "mixed form: the direct Volterra sum is FP64-only; use GEMM or FFT";
        return RBG_ERR_UNSUPPORTED;
    }
    const int N = plan.N;
    const int Np = (N + kChunk - 1) / kChunk * kChunk;
    int backend = o.conv;
    if (backend == RBG_CONV_AUTO) backend = (Np <= kMaxNpMulti) ? RBG_CONV_GEMM : RBG_CONV_FFT;
    if (backend == RBG_CONV_GEMM && Np > kMaxNpMulti) {
        err = "mixed GEMM form supports N <= 4096 (eight passes over 128 x 512 FP32 TMEM columns)";
        return RBG_ERR_UNSUPPORTED;
    }
    if (backend == RBG_CONV_FFT && N > 4096) {
        err = "mixed FFT backend supports N <= 4096 (two 8192-point buffers in shared memory)";
        return RBG_ERR_UNSUPPORTED;
    }
    job = MixedJob();
    job.mc = mc;
    const int ns = mc ? 3 : 2;
    job.backend = backend;
    job.N = N;
    job.n_vol = (int)plan.vols.size();
    job.n_vg = (int)plan.vgs.size();
    job.split = o.split;
    job.sms = dv.sms;
    if (o.split != RBG_SPLIT_BF16X3 && o.split != RBG_SPLIT_F16X3 && o.split != RBG_SPLIT_TF32X2) {
        err = "unknown split";
        return RBG_ERR_ARG;
    }
    // split kind of the kernels: 0 FP16x3, 1 BF16x3, 2 TF32 with one compensation term
    const int sk = split_kind(o.split);
    const bool tf32 = sk == 2;
    const int optin = dv.optin;
    int tcols = 32;
    while (tcols < std::min(Np, kPassCols)) tcols <<= 1;
    // variance groups per GEMM launch: as many as fit two pipeline stages
    int ng_cap = kMaxG;
    if (backend == RBG_CONV_GEMM) {
        while (ng_cap > 1 && smem_layout(Np, 2, ng_cap, 0, ns, tf32).total > optin) --ng_cap;
        if (smem_layout(Np, 2, ng_cap, 0, ns, tf32).total > optin) {
            err = "mixed kernel shared memory does not fit";
            return RBG_ERR_UNSUPPORTED;
        }
    }

    size_t off = 256;  // the error word lives at offset 0
    job.off_err = 0;
    const double log2e = 1.4426950408889634;
    for (int v = 0; v < job.n_vol; ++v) {
        const VolGroup& vol = plan.vols[v];
        for (int g0 = vol.vg_begin; g0 < vol.vg_end; g0 += ng_cap) {
            const int ng = std::min(ng_cap, vol.vg_end - g0);
            MixedLaunch r;
            std::memset(&r.args, 0, sizeof(r.args));
            MixedArgs& A = r.args;
            A.N = N;
            A.Np = Np;
            A.nc = Np / kChunk;
            A.np = (backend == RBG_CONV_GEMM) ? (Np + kPassCols - 1) / kPassCols : 1;
            A.n0 = (backend == RBG_CONV_GEMM && Np > kPassCols) ? (Np - kPassCols * (A.np - 1)) / kChunk : 0;
            A.n_g = ng;
            A.g0 = g0;
            A.tmem_cols = tcols;
            A.stages = 3;
            A.a1 = (float)vol.a1;
            A.a2 = (float)vol.a2;
            A.xi = (float)plan.xi;
            A.sqrt_xi = (float)std::sqrt(plan.xi);
            for (int g = 0; g < ng; ++g) {
                const VGroup& G = plan.vgs[g0 + g];
                A.alpha[g] = (float)(0.5 * G.eta * G.scale * log2e);  // halved: the epilogue forms sqrt(v)
                A.dt[g] = (float)G.dt;
                A.sdt[g] = (float)G.sdt;
                A.nsteps[g] = G.nsteps;
            }
            if (backend == RBG_CONV_GEMM) {
                r.off_strip = off;
                off += (size_t)strip_bytes_sk(Np, tf32);
                off = (off + 255) / 256 * 256;
            } else {
                A.logL = fft_log2_len(N);
                A.L = 1 << A.logL;
                if (fft_smem_bytes(N, ng, ns) > (size_t)optin) {
                    err = "mixed FFT kernel shared memory does not fit";
                    return RBG_ERR_UNSUPPORTED;
                }
                r.off_spec = off;
                off += (size_t)A.L * 8;
                off = (off + 255) / 256 * 256;
            }
            r.off_beta = off;
            off += (size_t)ng * Np * 4;
            off = (off + 255) / 256 * 256;
            int n_o = 0;
            for (const OutMap& om : plan.outs)
                if (om.vg >= g0 && om.vg < g0 + ng) ++n_o;
            A.n_o = n_o;
            A.n_out_total = (int)plan.outs.size();
            r.off_otab = off;
            off += (size_t)n_o * 16;
            off = (off + 255) / 256 * 256;
            r.off_oidx = off;
            off += (size_t)n_o * 4;
            off = (off + 255) / 256 * 256;
            job.launches.push_back(r);
        }
    }
    // fuse the payoffs into the GEMM path kernel when every launch has few outputs
    // Pricing the payoffs inside the path kernel's epilogue (RBG_FUSE_PAYOFFS)
    // measured slower than the separate FP32 payoff kernel on GB300 (6.84
    // against 6.14 ms per step at N = 512, 2^22 paths, 21 strikes): the
    // per-path Black-Scholes evaluations take issue slots the producer warps,
    // which set the kernel's pace, need.
    job.fused = RBG_FUSE_PAYOFFS && (backend == RBG_CONV_GEMM) && !mc;
    for (const MixedLaunch& r : job.launches)
        if (r.args.n_o > kMixedMaxFused || smem_layout(Np, 2, r.args.n_g, r.args.n_o, 2, tf32).total > optin)
            job.fused = false;
    // Pass mode 3 replaces the redrawing two-pass schedule for the 16-bit splits
    // and the RT estimator where two stages (three where they fit) and the
    // cached-tile slots fit.
    job.pmode = backend == RBG_CONV_GEMM ? pass_mode(Np) : 0;
    if (RBG_PASS3 && tile_cache && job.pmode == 1 && !tf32 && !mc) {
        bool fits = true;
        for (const MixedLaunch& r : job.launches)
            fits = fits &&
                   smem_layout(Np, 2, r.args.n_g, job.fused ? r.args.n_o : 0, ns, false, kCSlots).total <= optin;
        if (fits) job.pmode = 3;
    }
    for (MixedLaunch& r : job.launches) {
        MixedArgs& A = r.args;
        const int no = job.fused ? A.n_o : 0;
        A.stages = (smem_layout(Np, 3, A.n_g, no, ns, tf32).total <= optin) ? 3 : 2;
        if (backend == RBG_CONV_GEMM && smem_layout(Np, A.stages, A.n_g, no, ns, tf32).total > optin) {
            err = "mixed kernel shared memory does not fit";
            return RBG_ERR_UNSUPPORTED;
        }
        r.stages_pm1 = A.stages;
        if (job.pmode == 3) {
            A.np = (Np + kHalfCols - 1) / kHalfCols;
            A.n0 = (Np - kHalfCols * (A.np - 1)) / kChunk;
            A.ncache = A.np >= 3 ? A.n0 + kHalfCols / kChunk * (A.np - 3) : 0;
            A.stages = smem_layout(Np, 3, A.n_g, no, ns, false, kCSlots).total <= optin ? 3 : 2;
        }
    }
    if (backend == RBG_CONV_FFT) {
        job.off_tw = off;
        off += (size_t)(1 << fft_log2_len(N)) * 8;
        off = (off + 255) / 256 * 256;
    }
    std::vector<unsigned char>& ws = job.host_ws;
    ws.assign(off, 0);
    for (const MixedLaunch& r : job.launches) {
        const MixedArgs& A = r.args;
        const int vol = plan.vgs[A.g0].vol;
        if (backend == RBG_CONV_GEMM)
            build_strip(plan.gamma.data() + (size_t)vol * N, N, Np, sk, ws.data() + r.off_strip);
        else
            fft_tables(plan.gamma.data() + (size_t)vol * N, N, A.logL, (float*)(ws.data() + r.off_spec),
                       (float*)(ws.data() + job.off_tw));
        {
            float* ot = (float*)(ws.data() + r.off_otab);
            int* oi = (int*)(ws.data() + r.off_oidx);
            int q = 0;
            for (size_t i = 0; i < plan.outs.size(); ++i) {
                const OutMap& om = plan.outs[i];
                if (om.vg < A.g0 || om.vg >= A.g0 + A.n_g) continue;
                ot[4 * q + 0] = (float)om.rho;
                ot[4 * q + 1] = (float)om.K;
                ot[4 * q + 2] = (float)std::log(om.K);
                ot[4 * q + 3] = (float)(om.vg - A.g0);
                oi[q] = (int)i;
                ++q;
            }
        }
        float* beta = (float*)(ws.data() + r.off_beta);
        for (int g = 0; g < A.n_g; ++g) {
            // the group's forward variance: the plan's, or the tuple's own in the control-variate form
            const double lnxi = std::log(plan.vgs[A.g0 + g].xi);
            for (int j = 0; j < Np; ++j) {
                const double cj = (j < N) ? plan.comp[(size_t)(A.g0 + g) * N + j] : 0.0;
                beta[(size_t)g * Np + j] = (float)(0.5 * (cj - lnxi) * log2e);
            }
        }
    }
    job.workspace_bytes = off;
    if (job.pmode == 3) {
        // the A-tile cache: ncache tiles per CTA, not part of the uploaded image
        job.off_acache = (off + 1023) / 1024 * 1024;
        job.workspace_bytes = job.off_acache + (size_t)job.sms * job.launches[0].args.ncache * kStageA;
    }
    // batch: float2 per (variance group, path) within 1 GiB
    int64_t cap = ((int64_t)1 << 30) / (8 * (int64_t)std::max(1, job.n_vg));
    cap = std::max<int64_t>(kTileM, cap / kTileM * kTileM);
    if (max_batch > 0) cap = std::min<int64_t>(cap, std::max<int64_t>(kTileM, max_batch / kTileM * kTileM));
    job.batch = std::min<int64_t>(M, cap);
    return RBG_OK;
}

// The image is pageable host memory: the copy stages it before returning, so
// the caller may release it at once.
int mixed_upload(const MixedJob& job, void* ws, cudaStream_t st, std::string& err)
{
    if (cudaMemcpyAsync(ws, job.host_ws.data(), job.host_ws.size(), cudaMemcpyHostToDevice, st) != cudaSuccess) {
        cudaGetLastError();
        err = "mixed workspace upload failed";
        return RBG_ERR_CUDA;
    }
    return RBG_OK;
}

int mixed_part_rows(const MixedJob& job, int64_t B)
{
    const int64_t ntiles = (B + kTileM - 1) / kTileM;
    return (int)std::min<int64_t>(ntiles, job.sms);
}

// The path kernel of a (split, estimator, normal source) for pass mode pm.
// Sobol' normals run up to two passes (N <= 1024; mixed_launch rejects more).
template <int SK, bool MC, int SRC>
static void (*gemm_kernel_pm(int pm))(MixedArgs)
{
    if constexpr (SK != 2 && !MC && SRC == 0)
        if (pm == 3) return k_mixed_gemm<SK, 3, false, 0>;
    if constexpr (SRC == 1)
        return pm == 0 ? k_mixed_gemm<SK, 0, MC, SRC> : k_mixed_gemm<SK, 1, MC, SRC>;
    else
        return pm == 0 ? k_mixed_gemm<SK, 0, MC, SRC>
                       : (pm == 1 ? k_mixed_gemm<SK, 1, MC, SRC> : k_mixed_gemm<SK, 2, MC, SRC>);
}

// The path kernel of a (split kind, estimator, normal source) for pass mode pm.
template <bool MC, int SRC>
static void (*gemm_kernel(int sk, int pm))(MixedArgs)
{
    return sk == 0 ? gemm_kernel_pm<0, MC, SRC>(pm)
                   : (sk == 1 ? gemm_kernel_pm<1, MC, SRC>(pm) : gemm_kernel_pm<2, MC, SRC>(pm));
}

int mixed_launch(const MixedJob& job, void* ws, uint64_t seed, int64_t path0, int64_t B, void* ivb,
                 cudaStream_t st, std::string& err, float* dbg_w, float* dbg_x, double* part,
                 unsigned long long* prof, float* ivq, const double* ext)
{
    if (ext && (job.sob || job.fused)) {
        err = "caller normals run with the separate payoff kernels and without Sobol' normals";
        return RBG_ERR_UNSUPPORTED;
    }
    if (job.mc && !ivq) {
        err = "plain Monte Carlo launch without an IsvdWp buffer";
        return RBG_ERR_ARG;
    }
    if (job.sob && (job.mc || job.backend != RBG_CONV_GEMM || job.N > kMaxNp)) {
        err = "Sobol' normals in the mixed form need the RT estimator and the GEMM backend with N <= 1024";
        return RBG_ERR_UNSUPPORTED;
    }
    unsigned char* base = (unsigned char*)ws;
    for (const MixedLaunch& r : job.launches) {
        MixedArgs A = r.args;
        const size_t li = (size_t)(&r - job.launches.data());
        const bool over = li < job.table_dev.size() && job.table_dev[li];
        A.strip = over ? (const unsigned char*)job.table_dev[li] : base + r.off_strip;
        A.beta = (const float*)(base + r.off_beta);
        A.spec = over ? (const float2*)job.table_dev[li] : (const float2*)(base + r.off_spec);
        A.otab = (const float4*)(base + r.off_otab);
        A.oidx = (const int*)(base + r.off_oidx);
        A.part = part;
        A.prof = prof;
        if (!job.fused || !part) A.n_o = 0;
        A.tw = (const float2*)(base + job.off_tw);
        A.ivb = (float2*)ivb;
        A.ivq = ivq;
        A.err = (unsigned int*)(base + job.off_err);
        A.dbg_w = dbg_w;
        A.dbg_x = dbg_x;
        A.sob = job.sob;
        A.ext = ext;
        mixed_set_seed(A, seed);
        A.path0 = path0;
        A.B = B;
        int pm = job.backend == RBG_CONV_GEMM ? pass_mode(A.Np) : 0;
        if (job.pmode == 3) {
            if (!ext && !job.sob) {
                pm = 3;
                A.acache = base + job.off_acache;
            } else {
                // Sobol' or caller normals: the two-pass kernel
                A.np = 2;
                A.n0 = (A.Np - kPassCols) / kChunk;
                A.stages = r.stages_pm1;
            }
        }
        const int smem = smem_layout(A.Np, A.stages, A.n_g, A.n_o, job.mc ? 3 : 2, job.split == RBG_SPLIT_TF32X2,
                                     pm == 3 ? kCSlots : 0)
                             .total;
        const int64_t ntiles = (B + kTileM - 1) / kTileM;
        const int grid = (int)std::min<int64_t>(ntiles, job.sms);
        cudaError_t e;
        if (job.backend == RBG_CONV_FFT) {
            e = launch_mixed_fft(A, job.sms, st);
        } else {
            const int sk = split_kind(job.split);
            void (*kern)(MixedArgs);
            if (job.sob)
                kern = gemm_kernel<false, 1>(sk, pm);
            else if (ext)
                kern = job.mc ? gemm_kernel<true, 2>(sk, pm) : gemm_kernel<false, 2>(sk, pm);
            else
                kern = job.mc ? gemm_kernel<true, 0>(sk, pm) : gemm_kernel<false, 0>(sk, pm);
            e = allow_max_smem(kern);
            // the multi-pass modes add a second MMA-issuing warp
            if (e == cudaSuccess) kern<<<grid, pm > 0 ? kThreads + 32 : kThreads, smem, st>>>(A);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string("mixed kernel launch: ") + cudaGetErrorString(e);
            return RBG_ERR_CUDA;
        }
        count_launch();
    }
    return RBG_OK;
}

bool mixed_job_batchable(const MixedJob& job)
{
    return job.backend == RBG_CONV_GEMM && job.launches.size() == 1 && job.launches[0].args.Np <= kPassCols &&
           !job.mc && !job.fused && !job.sob;
}

size_t mixed_jobs_table_bytes(int n) { return sizeof(MixedArgs) * (size_t)n + sizeof(int64_t) * (size_t)(n + 1); }

int mixed_jobs_prepare(const std::vector<MixedJobRef>& jobs, void* table, unsigned int* err, int sms,
                       std::vector<unsigned char>& host_table, MixedArgs* launch_args, std::string& errmsg)
{
    const int n = (int)jobs.size();
    if (n < 1) {
        errmsg = "empty job table";
        return -1;
    }
    const int split = jobs[0].job->split;
    host_table.assign(mixed_jobs_table_bytes(n), 0);
    MixedArgs* args = (MixedArgs*)host_table.data();
    int64_t* tile0 = (int64_t*)(host_table.data() + sizeof(MixedArgs) * (size_t)n);
    int Np_max = 0, ng_max = 1, tcols = 32;
    tile0[0] = 0;
    for (int k = 0; k < n; ++k) {
        const MixedJobRef& r = jobs[k];
        if (!mixed_job_batchable(*r.job) || r.job->split != split) {
            errmsg = "job-table launch: every job needs one one-pass RT launch of the same split";
            return -1;
        }
        const MixedLaunch& L = r.job->launches[0];
        MixedArgs A = L.args;
        const unsigned char* base = (const unsigned char*)r.ws;
        const bool over = !r.job->table_dev.empty() && r.job->table_dev[0];
        A.strip = over ? (const unsigned char*)r.job->table_dev[0] : base + L.off_strip;
        A.beta = (const float*)(base + L.off_beta);
        A.ivb = (float2*)r.ivb;
        A.ivq = nullptr;
        A.err = err;
        A.otab = nullptr;
        A.oidx = nullptr;
        A.part = nullptr;
        A.prof = nullptr;
        A.spec = nullptr;
        A.tw = nullptr;
        A.sob = nullptr;
        A.ext = nullptr;
        A.dbg_w = nullptr;
        A.dbg_x = nullptr;
        A.n_o = 0;
        mixed_set_seed(A, r.seed);
        A.path0 = r.path0;
        A.B = r.B;
        A.jobs = nullptr;
        A.job_tile0 = nullptr;
        A.n_jobs = 0;
        args[k] = A;
        tile0[k + 1] = tile0[k] + (r.B + kTileM - 1) / kTileM;
        Np_max = std::max(Np_max, A.Np);
        ng_max = std::max(ng_max, A.n_g);
        tcols = std::max(tcols, A.tmem_cols);
    }
    DevInfo dv;
    if (!device_info(&dv)) {
        errmsg = "device attribute query failed";
        return -1;
    }
    const int optin = dv.optin;
    const bool tf32 = split == RBG_SPLIT_TF32X2;
    MixedArgs LA = args[0];
    LA.Np = Np_max;
    LA.nc = Np_max / kChunk;
    LA.n_g = ng_max;
    LA.tmem_cols = tcols;
    LA.stages = smem_layout(Np_max, 3, ng_max, 0, 2, tf32).total <= optin ? 3 : 2;
    if (smem_layout(Np_max, LA.stages, ng_max, 0, 2, tf32).total > optin) {
        errmsg = "job-table launch: shared memory does not fit";
        return -1;
    }
    LA.strip = nullptr;
    LA.beta = nullptr;
    LA.ivb = nullptr;
    LA.B = 0;
    LA.jobs = (const MixedArgs*)table;
    LA.job_tile0 = (const int64_t*)((const unsigned char*)table + sizeof(MixedArgs) * (size_t)n);
    LA.n_jobs = n;
    *launch_args = LA;
    return (int)std::min<int64_t>(tile0[n], sms);
}

int mixed_launch_jobs(const MixedArgs& A, int split, int grid, cudaStream_t st, std::string& errmsg)
{
    const int sk = split_kind(split);
    void (*kern)(MixedArgs) = sk == 0 ? k_mixed_gemm_jobs<0> : (sk == 1 ? k_mixed_gemm_jobs<1> : k_mixed_gemm_jobs<2>);
    const int smem = smem_layout(A.Np, A.stages, A.n_g, 0, 2, sk == 2).total;
    cudaError_t e = allow_max_smem(kern);
    if (e == cudaSuccess) {
        kern<<<grid, kThreads, smem, st>>>(A);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        errmsg = std::string("job-table kernel launch: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    count_launch();
    return RBG_OK;
}

// Loads the path and payoff kernels a serving loop may launch (CUDA loads a
// kernel's module lazily, on first use: a load in the middle of a request
// stream stalls that request's launch).
void mixed_preload()
{
    cudaFuncAttributes fa;
    void (*kerns[])(MixedArgs) = {
        k_mixed_gemm<0, 0, false>, k_mixed_gemm<0, 1, false>, k_mixed_gemm<0, 2, false>,
        k_mixed_gemm<1, 0, false>, k_mixed_gemm<1, 1, false>, k_mixed_gemm<1, 2, false>,
        k_mixed_gemm<2, 0, false>, k_mixed_gemm<2, 1, false>, k_mixed_gemm<2, 2, false>,
        k_mixed_gemm_jobs<0>, k_mixed_gemm_jobs<1>, k_mixed_gemm_jobs<2>};
    for (auto k : kerns) cudaFuncGetAttributes(&fa, k);
    cudaFuncGetAttributes(&fa, k_payoff_sums_f32<false>);
    cudaFuncGetAttributes(&fa, k_payoff_sums_f32_jobs);
    cudaGetLastError();
}

int mixed_check(const MixedJob& job, void* ws, cudaStream_t st, std::string& err)
{
    unsigned int word = 0;
    cudaError_t e = cudaMemcpyAsync(&word, (unsigned char*)ws + job.off_err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("mixed kernel failed: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    if (word != 0) {
        err = "mixed kernel: a bounded pipeline wait expired (site " + std::to_string(word) + ")";
        return RBG_ERR_TIMEOUT;
    }
    return RBG_OK;
}



}  // namespace rbg
