// pg_tc.cu -- tcgen05 (5th-generation tensor core) kernels for sm_103a.
//
// The fixed-end normal-mode transform T (P x P, DST-I, symmetric, T T = I) is
// the only dense contraction of the TI-PIMD step.  Here it runs on the tensor
// cores as a split-BF16 product with FP32 accumulation in tensor memory:
//     T X ~= T_hi X_hi + T_hi X_lo + T_lo X_hi,   v_hi = bf16(v), v_lo = bf16(v - v_hi)
// (relative error ~ 2^-17 per element).
//
// Two layouts.  The standalone transform (k_tc_transform) gives one CTA 128
// input columns, one thread per column: D[col][n] = sum_k X[col][k] T[n][k]
// (A = data written by the thread that owns the TMEM lane, B = T).  The TI step
// kernels (k_tc_g1, k_tc_g2) swap the roles: A = T (M = 128 beads or modes), B =
// a tile of 64 state columns (N = 64), so a TMEM lane holds one bead of all
// columns and two 256-thread CTAs fit on an SM.  K = 128 in 8 steps of 16,
// three MMAs per step, one commit per launch.
//
// State lives in HBM/L2 as FP32 [ring][dof][P] (q, pi, x, F), the same layout
// as the SIMT kernels, so state read-out and checkpoints are shared.
#include <cuda_bf16.h>

#include <algorithm>

#include <cstdio>
#include <mutex>
#include <vector>

#include "pg_internal.h"

namespace pg {

void build_transmatrix(int P, std::vector<double> &T);

namespace {

constexpr int kP = 128;            // beads (= modes = MMA K)
constexpr int kRows = 128;         // ring-dof columns per CTA (MMA M)
constexpr int kOpBytes = kRows * kP * 2;  // one bf16 operand image: 32 KB
constexpr uint32_t kLBO = 128;     // byte offset between K-adjacent 8x16B core matrices
constexpr uint32_t kSBO = 2048;    // byte offset between M/N-adjacent 8-row groups
constexpr long long kSpinLimit = 20000000LL;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

// Byte offset of element (row, k) in a K-major, no-swizzle core-matrix image.
__host__ __device__ __forceinline__ uint32_t op_offset(int row, int k) {
    return (uint32_t)((row >> 3) * kSBO + (k >> 3) * kLBO + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// 64-bit shared-memory matrix descriptor (no swizzle, K-major).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(kLBO >> 4) << 16;
    d |= (uint64_t)(kSBO >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for sm_100-family tcgen05
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, K-major, M = 128, N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: gives up (returns false) after ~2 s of wall time.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint64_t t0 = globaltimer_ns();
    for (long long i = 0; i < kSpinLimit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 63) == 63 && globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
    return false;
}
// Non-blocking test of a phase (mbarrier.test_wait never suspends the thread).
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait bounded by a deadline: it gives up once limit_ns have passed since t0
// (the kernel's start), and the deadline is checked before each test, so a
// limit of 0 gives up at the first wait whatever the state of the phase.  A
// caller whose wait gives up must still let the operation it waited for finish
// (mbar_wait, bounded by the fixed limit) before the CTA frees tensor memory or
// exits.
__device__ __forceinline__ bool mbar_wait_until(uint64_t *bar, uint32_t parity, uint64_t t0, uint64_t limit_ns) {
    for (long long i = 0; i < kSpinLimit; i++) {
        if (globaltimer_ns() - t0 >= limit_ns) return false;
        if (mbar_test_wait(bar, parity)) return true;
    }
    return false;
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

#define PG_R32(v)                                                                                       \
    "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),     \
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),       \
        "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),     \
        "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),     \
        "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
#define PG_W32(v)                                                                                         \
    "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),  \
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]), \
        "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]), \
        "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

// 32 consecutive FP32 columns of this thread's TMEM lane.  The load and its
// wait are one asm statement, so no use of the outputs can be scheduled
// between them.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&out)[32]) {
    uint32_t v[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
        "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : PG_R32(v)
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) out[i] = __uint_as_float(v[i]);
}
// N = 8 or 16 consecutive FP32 columns of this thread's TMEM lane.
template <int N>
__device__ __forceinline__ void tmem_ldn(uint32_t taddr, float (&out)[N]) {
    static_assert(N == 8 || N == 16 || N == 32, "TMEM load width");
    if constexpr (N == 32) {
        tmem_ld32(taddr, out);
    } else if constexpr (N == 16) {
        uint32_t v[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            "tcgen05.wait::ld.sync.aligned;"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr)
            : "memory");
#pragma unroll
        for (int i = 0; i < 16; i++) out[i] = __uint_as_float(v[i]);
    } else {
        uint32_t v[8];
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                     "tcgen05.wait::ld.sync.aligned;"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                     : "r"(taddr)
                     : "memory");
#pragma unroll
        for (int i = 0; i < 8; i++) out[i] = __uint_as_float(v[i]);
    }
}
// 8 FP32 values into consecutive TMEM columns of this thread's lane; the
// store and its wait are one asm statement (a later tcgen05.ld of the same
// columns by this thread sees them).
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n"
        "tcgen05.wait::st.sync.aligned;" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
        : "memory");
}
// 32 FP32 values into consecutive TMEM columns of this thread's lane; store and
// wait in one asm statement, as tmem_st8.
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&f)[32]) {
    uint32_t v[32];
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __float_as_uint(f[i]);
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
        "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};\n"
        "tcgen05.wait::st.sync.aligned;" ::"r"(taddr),
        PG_W32(v)
        : "memory");
}
// Two groups of 8 consecutive FP32 columns (at ta and tb) of this thread's lane:
// both loads, then one wait, in one asm statement.
__device__ __forceinline__ void tmem_ld8x2(uint32_t ta, uint32_t tb, float (&a)[8], float (&b)[8]) {
    uint32_t v[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%16];\n"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%17];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(ta), "r"(tb)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; i++) {
        a[i] = __uint_as_float(v[i]);
        b[i] = __uint_as_float(v[8 + i]);
    }
}
// Write 32 FP32 values of row `row`, K = k0..k0+31, into the hi / lo operand images.
__device__ __forceinline__ void write_split32(unsigned char *Ahi, unsigned char *Alo, int row, int k0,
                                              const float (&v)[32]) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            float a0 = v[8 * c + 2 * e], a1 = v[8 * c + 2 * e + 1];
            __nv_bfloat16 h0 = __float2bfloat16_rn(a0), h1 = __float2bfloat16_rn(a1);
            float r0 = a0 - __bfloat162float(h0), r1 = a1 - __bfloat162float(h1);
            __nv_bfloat162 hh;
            hh.x = h0;
            hh.y = h1;
            h[e] = *reinterpret_cast<uint32_t *>(&hh);
            l[e] = pack_bf16(r0, r1);
        }
        uint32_t off = op_offset(row, k0 + 8 * c);
        *reinterpret_cast<uint4 *>(Ahi + off) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(Alo + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
}

// D(tmem col dcol) = A * B^T over K = 128, split-BF16 (3 products per K step).
__device__ __forceinline__ void issue_gemm(uint32_t tmem, uint32_t dcol, uint32_t a_hi, uint32_t a_lo,
                                           uint32_t b_hi, uint32_t b_lo, uint64_t *bar) {
#pragma unroll
    for (int ks = 0; ks < kP / 16; ks++) {
        uint32_t koff = (uint32_t)ks * 2 * kLBO;
        uint64_t ah = make_desc(a_hi + koff), al = make_desc(a_lo + koff);
        uint64_t bh = make_desc(b_hi + koff), bl = make_desc(b_lo + koff);
        mma_bf16(tmem + dcol, ah, bh, ks > 0 ? 1u : 0u);
        mma_bf16(tmem + dcol, ah, bl, 1u);
        mma_bf16(tmem + dcol, al, bh, 1u);
    }
    mma_commit(bar);
}

struct TcShared {
    uint64_t mma_bar;
    uint64_t tma_bar;
    uint64_t mma_bar2;  // blocked GEMM: second MMA-completion barrier (T_lo products)
    uint64_t tma_bar2;  // blocked GEMM: second copy barrier (T_lo half)
    uint32_t tmem_slot;
    int32_t err;
};

// Dynamic shared memory: [T_hi | T_lo | A_hi | A_lo] (32 KB each, 1024-aligned),
// then per-atom mode coefficients, then TcShared.
constexpr int kSmemOps = 4 * kOpBytes;

__device__ __forceinline__ unsigned char *align1k(unsigned char *p) {
    return reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~(uintptr_t)1023);
}

// Load the split-BF16 transform image (64 KB) with bulk async copies.
__device__ __forceinline__ void load_transform(unsigned char *Thi, const unsigned char *gT, TcShared *sh) {
    if (threadIdx.x == 0) {
        mbar_expect_tx(&sh->tma_bar, 2 * kOpBytes);
#pragma unroll
        for (int i = 0; i < 4; i++) bulk_g2s(Thi + i * 16384, gT + i * 16384, 16384, &sh->tma_bar);
    }
}

// ---------------------------------------------------------------- standalone transform
// out[c][:] = T in[c][:] for 128 columns per CTA (used by pg_nm_transform, P = 128).
// The waits for the T copy and for the GEMM share a deadline of wait_ns (the
// context's wait limit) from the kernel's start.  A wait that gives up records
// the error and then waits (bounded by the fixed 2 s limit) for that copy or
// GEMM to finish, so that no asynchronous write into shared or tensor memory
// outlives the CTA's deallocation and exit; the GEMM is not issued after a
// failed copy wait.
__global__ void __launch_bounds__(128, 1) k_tc_transform(const unsigned char *__restrict__ gT,
                                                          const double *__restrict__ in,
                                                          double *__restrict__ out, int64_t ncol,
                                                          int32_t *__restrict__ err, uint64_t wait_ns) {
    const uint64_t t_start = globaltimer_ns();
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    unsigned char *Thi = base, *Tlo = base + kOpBytes, *Ahi = base + 2 * kOpBytes, *Alo = base + 3 * kOpBytes;
    TcShared *sh = reinterpret_cast<TcShared *>(base + kSmemOps);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&sh->mma_bar, 1);
        mbar_init(&sh->tma_bar, 1);
        sh->err = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (warp == 0) tmem_alloc(&sh->tmem_slot, 128);
    load_transform(Thi, gT, sh);
    // rows = columns of the input
    const int64_t c = (int64_t)blockIdx.x * kRows + tid;
    for (int k0 = 0; k0 < kP; k0 += 32) {
        float v[32];
#pragma unroll
        for (int i = 0; i < 32; i++) v[i] = c < ncol ? (float)in[c * kP + k0 + i] : 0.f;
        write_split32(Ahi, Alo, tid, k0, v);
    }
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = sh->tmem_slot;
    if (tid == 0) {
        if (mbar_wait_until(&sh->tma_bar, 0, t_start, wait_ns)) {
            issue_gemm(tmem, 0, smem_u32(Ahi), smem_u32(Alo), smem_u32(Thi), smem_u32(Tlo), &sh->mma_bar);
        } else {
            sh->err = 1;
            mbar_wait(&sh->tma_bar, 0);  // the copy lands before the CTA may exit
        }
    }
    __syncthreads();
    bool issued = sh->err == 0;
    if (issued && !mbar_wait_until(&sh->mma_bar, 0, t_start, wait_ns)) {
        atomicOr(&sh->err, 2);
        mbar_wait(&sh->mma_bar, 0);  // the GEMM finishes before TMEM is read or freed
    }
    tc_after();
    __syncthreads();
    if (sh->err == 0) {
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
        for (int n0 = 0; n0 < kP; n0 += 32) {
            float v[32];
            tmem_ld32(lane_addr + (uint32_t)n0, v);
            if (c < ncol)
#pragma unroll
                for (int i = 0; i < 32; i++) out[c * kP + n0 + i] = (double)v[i];
        }
    } else if (tid == 0) {
        atomicOr(err, sh->err);
    }
    tc_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 128);
}

// Writes the split-BF16 image of T (P = 128, K-major core-matrix layout) on the
// device: one thread per (n, k) element.
__global__ void k_build_split_image(unsigned char *img) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kP * kP) return;
    const int n = e / kP, k = e - n * kP;
    double v = sin((double)((n + 1) * (k + 1)) * kPiRef / (double)(kP + 1)) * sqrt(2.0 / (double)(kP + 1));
    __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
    __nv_bfloat16 lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
    const uint32_t off = op_offset(n, k);
    *reinterpret_cast<__nv_bfloat16 *>(img + off) = hi;
    *reinterpret_cast<__nv_bfloat16 *>(img + kOpBytes + off) = lo;
}

// ---------------------------------------------------------------- TI step on the tensor cores
// k_tc_step runs up to 50 MD steps per launch (two split-BF16 GEMMs per column
// tile and step with the forces in between); one final launch per advance
// (k_tc_final) writes the positions and the estimator of the last step.  The
// ring state stays resident in L2 (and q in tensor memory within a launch);
// the launches of an advance are replayed from one captured CUDA graph,
// followed by one step-counter add.
struct TcArgs {
    int64_t nrings;
    int nd, ndim, natom;
    float dt;
    int64_t imin;
    const unsigned char *gT;  // split-BF16 transform image (64 KB)
    const float *coef;        // natom x P x 8: rA rB rC rD ou_a ou_s
    const double *mass;       // natom
    const double *avec;       // nd
    const double *bvec;       // nlambda*nd
    const double *dbdl;       // nlambda*nd
    const int32_t *ringlam;
    const uint64_t *ringseed;
    const uint32_t *ringstream;
    float *q, *pi, *x;        // [ring][dof][P]
    RingAcc *acc;
    // per state column (ring-major, nrings * nd), built once per batch by k_tc_cols
    const float *cxa, *cxs;   // spring line x*_m = xa + xs (m + 1)
    const uint64_t *cseed;
    const uint32_t *cstream;
    const int32_t *cjdof;     // dof index of the column within its ring
    const double *cwest;      // estimator weight mass * db/dlambda
    const float *fold;        // P x 8: K11 K12 N1 K11 dt | K21 K22 N2 K21 dt (kick + rotation + OU + rotation)
    const int64_t *step0;     // step counter at the start of the advance (not written by these kernels)
    int64_t sofs;             // this launch's step offset within the advance
    int do_est;               // accumulate the estimator of step s-1
    int nsub;                 // k_tc_step: MD steps sofs .. sofs + nsub - 1 in this launch
    int32_t *err;
    // PES parameters (FP32)
    float wc[12];
    int nwell;
    float a0, b0;
    int pow10;
    float H, x0;
};

// ---------------------------------------------------------------- column tiles
// The TI step kernels work on tiles of kNc = 64 ring-dof columns with 256
// threads (8 warps), two CTAs per SM.  A split-BF16 GEMM
//     D[m][c] = sum_k T[m][k] X[c][k]     (M = 128 beads or modes, N = 64, K = 128)
// takes T as the A operand (the bulk-copied image) and a tile X of FP32 state
// columns, split by the CTA's threads, as the B operand.  TMEM lane m then
// holds bead (or mode) m of all 64 columns: warp w reads lane quadrant w % 4
// and column half w / 4, so every epilogue access of a warp covers 32
// consecutive beads of one column (128 contiguous bytes), and the x / y
// columns of a ring (2r, 2r+1) sit in the same thread.  Tiles hold whole rings
// (64 is a multiple of the 1 or 2 dofs of the surfaces this form runs).
constexpr int kNc = 64;
constexpr int kTileThreads = 256;
constexpr int kGrp = 8;  // columns per TMEM load in the epilogues
// B operand layout: K-major core matrices (8 rows x 16 bytes) as for T, but
// K-adjacent core matrices kXLbo = 160 bytes apart (32 bytes of padding), so
// that warp stores of one column's 32 beads (4 core matrices) and of the next
// column (16 bytes further) fall in distinct banks.
constexpr uint32_t kXLbo = 160;
constexpr uint32_t kXSbo = 16 * kXLbo;                                 // 8-row groups: 2560 bytes
constexpr int kXPlane = (kNc / 8) * (int)kXSbo;                        // one bf16 plane: 20 KB
constexpr int kTileSmemOps = 2 * kOpBytes + 2 * kXPlane;               // T hi/lo + X hi/lo: 104 KB
constexpr uint32_t kIdescN64 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kNc >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);

__host__ __device__ __forceinline__ uint32_t x_offset(int row, int k) {
    return (uint32_t)((row >> 3) * kXSbo + (k >> 3) * kXLbo + (row & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ uint64_t make_desc_x(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(kXLbo >> 4) << 16;
    d |= (uint64_t)(kXSbo >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Per-column values staged in shared memory by the CTA.
struct TileAux {
    float4 msc[kNc];     // the column's atom mass factors (m, sqrt m, 1 / m, 1 / sqrt m)
    float xa[kNc];       // spring-line start a_j
    float xs[kNc];       // spring-line slope (b_j - a_j) / (P + 1)
    float xP[kNc];       // bead-P position for the estimator
    uint64_t seed[kNc];  // Philox key of the column's ring
    uint32_t stream[kNc];
    int32_t jdof[kNc];   // the column's dof index within its ring
    int32_t atom[kNc];   // the column's atom
};

// Per-column values of one chunk of the step kernel, copied in from the
// column table (cp.async, one chunk ahead).
struct StepStage {
    float xa[kNc], xs[kNc];
    uint64_t seed[kNc];
    double west[kNc];
    uint32_t stream[kNc];
    int32_t jdof[kNc];
};
struct StepAux {
    float xP[kNc];  // bead-P positions for the estimator
    StepStage stg[2];
};

__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Bulk prefetch of [p, p + bytes) into L2 (a hint: p 16-byte aligned, bytes a
// multiple of 16).
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
// Programmatic dependent launch: both are no-ops for a launch without the
// programmatic-serialization attribute.
__device__ __forceinline__ void griddep_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Thread t < kNc of the CTA: column col0 + t of the table into sg (zeros for
// t >= nvalid).  async: cp.async (the caller commits and waits), else loads.
__device__ __forceinline__ void stage_columns(StepStage *sg, const TcArgs &a, int64_t col0, int nvalid, bool async) {
    const int t = threadIdx.x;
    if (t < nvalid) {
        const int64_t c = col0 + t;
        if (async) {
            cp_async4(&sg->xa[t], a.cxa + c);
            cp_async4(&sg->xs[t], a.cxs + c);
            cp_async8(&sg->seed[t], a.cseed + c);
            cp_async8(&sg->west[t], a.cwest + c);
            cp_async4(&sg->stream[t], a.cstream + c);
            cp_async4(&sg->jdof[t], a.cjdof + c);
        } else {
            sg->xa[t] = a.cxa[c];
            sg->xs[t] = a.cxs[c];
            sg->seed[t] = a.cseed[c];
            sg->west[t] = a.cwest[c];
            sg->stream[t] = a.cstream[c];
            sg->jdof[t] = a.cjdof[c];
        }
    } else {
        sg->xa[t] = 0.f;
        sg->xs[t] = 0.f;
        sg->seed[t] = 0;
        sg->west[t] = 0.0;
        sg->stream[t] = 0;
        sg->jdof[t] = 0;
    }
}

__device__ __forceinline__ void mma_bf16_n64(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(kIdescN64), "r"(acc)
        : "memory");
}

// Splits 8 FP32 values into one 16-byte row of the hi and of the lo plane.
__device__ __forceinline__ void split8(const float (&v)[8], uint4 &hi, uint4 &lo) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * e]), h1 = __float2bfloat16_rn(v[2 * e + 1]);
        float r0 = v[2 * e] - __bfloat162float(h0), r1 = v[2 * e + 1] - __bfloat162float(h1);
        __nv_bfloat162 hh;
        hh.x = h0;
        hh.y = h1;
        h[e] = *reinterpret_cast<uint32_t *>(&hh);
        l[e] = pack_bf16(r0, r1);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// One-time set-up of a CTA: barriers, the T image by bulk copy (completes
// tma_bar phase 0), kNc TMEM columns.  Returns the TMEM base address.
__device__ __forceinline__ uint32_t tile_setup(unsigned char *base, TcShared *sh, const unsigned char *gT,
                                               uint32_t ncols = kNc) {
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&sh->mma_bar, 1);
        mbar_init(&sh->tma_bar, 1);
        sh->err = 0;
        fence_barrier_init();
    }
    __syncthreads();
    load_transform(base, gT, sh);
    if (warp == 0) {
        __syncwarp();
        tmem_alloc(&sh->tmem_slot, ncols);
    }
    tc_before();
    __syncthreads();
    tc_after();
    return sh->tmem_slot;
}

// The tile X[c][k] = src[c * P + k] (zero for c >= nvalid) split into the B
// operand.  Ends with a CTA barrier after which the operand (and anything the
// CTA wrote to shared memory before the call) is visible to the tensor core.
__device__ __forceinline__ void tile_load(unsigned char *base, const float *src, int nvalid) {
    unsigned char *Xhi = base + 2 * kOpBytes, *Xlo = Xhi + kXPlane;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // Warp w fills rows 8w..8w+7.  Lane: row 8w + lane % 8, K chunks
    // 8 (4 it + lane / 8): the 8 lanes of one chunk write one core matrix.
    const int c = 8 * warp + (lane & 7);
    const bool v = c < nvalid;
    const float *row = src + (size_t)(v ? c : 0) * kP;
    float4 w[8];
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int k0 = 8 * (4 * it + (lane >> 3));
        w[2 * it] = v ? __ldg(reinterpret_cast<const float4 *>(row + k0)) : make_float4(0.f, 0.f, 0.f, 0.f);
        w[2 * it + 1] = v ? __ldg(reinterpret_cast<const float4 *>(row + k0 + 4)) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int k0 = 8 * (4 * it + (lane >> 3));
        const float e8[8] = {w[2 * it].x,     w[2 * it].y,     w[2 * it].z,     w[2 * it].w,
                             w[2 * it + 1].x, w[2 * it + 1].y, w[2 * it + 1].z, w[2 * it + 1].w};
        uint4 hi, lo;
        split8(e8, hi, lo);
        const uint32_t off = x_offset(c, k0);
        *reinterpret_cast<uint4 *>(Xhi + off) = hi;
        *reinterpret_cast<uint4 *>(Xlo + off) = lo;
    }
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
}

// Set-up and first tile in one (single-tile kernels).
__device__ __forceinline__ uint32_t tile_begin(unsigned char *base, TcShared *sh, const unsigned char *gT,
                                               const float *src, int nvalid) {
    const uint32_t tmem = tile_setup(base, sh, gT);
    tile_load(base, src, nvalid);
    return tmem;
}

// Thread 0 issues D = T X (3 split products per K step of 16) and commits it
// to mma_bar; wait_t: first wait for the bulk copy of T.  A failed wait sets
// the CTA error word instead of issuing.
__device__ __forceinline__ void tile_issue(unsigned char *base, TcShared *sh, uint32_t tmem, bool wait_t) {
    if (threadIdx.x != 0) return;
    if (sh->err) return;
    if (wait_t && !mbar_wait(&sh->tma_bar, 0)) {
        sh->err |= 1;
        return;
    }
    const uint32_t th = smem_u32(base), tl = th + kOpBytes, xh = th + 2 * kOpBytes, xl = xh + kXPlane;
    // descriptors of K step 0; step ks adds its byte offset / 16 to the start
    // address field (shared addresses stay below 2^18, so no carry leaves it)
    const uint64_t dth0 = make_desc(th), dtl0 = make_desc(tl), dxh0 = make_desc_x(xh), dxl0 = make_desc_x(xl);
#pragma unroll
    for (int ks = 0; ks < kP / 16; ks++) {
        const uint64_t ot = (uint64_t)(ks * 2 * kLBO / 16), ox = (uint64_t)(ks * 2 * kXLbo / 16);
        mma_bf16_n64(tmem, dth0 + ot, dxh0 + ox, ks > 0 ? 1u : 0u);
        mma_bf16_n64(tmem, dth0 + ot, dxl0 + ox, 1u);
        mma_bf16_n64(tmem, dtl0 + ot, dxh0 + ox, 1u);
    }
    mma_commit(&sh->mma_bar);
}

// Every thread waits for the GEMM of the given mbarrier phase; returns whether
// the accumulator is valid (CTA-uniform after the barrier).
__device__ __forceinline__ bool tile_wait(TcShared *sh, uint32_t parity) {
    __syncthreads();  // thread 0 has issued (or recorded an error)
    const bool issued = sh->err == 0;
    if (issued && !mbar_wait(&sh->mma_bar, parity)) atomicOr(&sh->err, 2);
    tc_after();
    __syncthreads();
    return sh->err == 0;
}

// Every thread waits for the GEMM of the given phase itself (no CTA barrier);
// a timeout is recorded in the CTA error word, which the caller checks after
// its next barrier.  The chunk structure keeps every thread within one phase
// of the barrier, so the parity cannot alias.
__device__ __forceinline__ void tile_wait_own(TcShared *sh, uint32_t parity) {
    if (!mbar_wait(&sh->mma_bar, parity)) atomicOr(&sh->err, 2);
    tc_after();
}

__device__ __forceinline__ void tile_release(TcShared *sh, uint32_t tmem, int32_t *gerr, uint32_t parity,
                                             uint32_t ncols = kNc) {
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0 && sh->err) atomicOr(gerr, sh->err);
    if (sh->err & 2) mbar_wait(&sh->mma_bar, parity);  // let an overdue MMA drain (bounded)
    tc_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tmem_dealloc(tmem, ncols);
    }
}

// Gradient of the FP32 six-well surface (mcmod_2dtest.f90:39-60) at the NR
// beads (x, y) = (xv[2r], xv[2r+1]) of one thread.  Wells are the outer loop so
// that the beads give NR independent chains per well; every bead still sums
// its wells in order k = 1..m.  POW10: a0 = 10 b0, so e^{-a0 u} = (e^{-b0 u})^10.
template <bool POW10, int NR>
__device__ __forceinline__ void grad_2d_n(const TcArgs &a, const float (&xv)[2 * NR], float (&gx)[NR],
                                          float (&gy)[NR]) {
#pragma unroll
    for (int r = 0; r < NR; r++) {
        gx[r] = 0.f;
        gy[r] = 0.f;
    }
    for (int k = 0; k < a.nwell; k++) {
        const float wx = a.wc[2 * k], wy = a.wc[2 * k + 1];
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const float dx = xv[2 * r] - wx, dy = xv[2 * r + 1] - wy;
            const float u = dx * dx + dy * dy;
            const float eb = __expf(-a.b0 * u);
            float ea;
            if (POW10) {
                const float e2 = eb * eb, e4 = e2 * e2, e8 = e4 * e4;
                ea = e8 * e2;
            } else {
                ea = __expf(-a.a0 * u);
            }
            const float cc = a.a0 * ea + a.b0 * eb;
            gx[r] += cc * dx;
            gy[r] += cc * dy;
        }
    }
}

// Packed FP32 pairs (two lanes per register pair, Blackwell f32x2 ops).
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(uint64_t v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t fmul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fadd2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ float ex2f(float v) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}

// The POW10 six-well gradient of grad_2d_n for NR beads (NR even), two rings
// per packed f32x2 operation: per well dx, dy, u = dx^2 + dy^2,
// eb = 2^(u (-b0 log2 e)), ea = eb^10, cc = a0 ea + b0 eb, g += cc d.
template <int NR, int NW = 0>  // NW > 0: the well count is NW (loop fully unrolled)
__device__ __forceinline__ void grad_2d_pow10_x2(const TcArgs &a, const float (&xv)[2 * NR], float (&gx)[NR],
                                                 float (&gy)[NR]) {
    static_assert(NR % 2 == 0, "pairs of rings");
    uint64_t X[NR / 2], Y[NR / 2], GX[NR / 2], GY[NR / 2];
#pragma unroll
    for (int r = 0; r < NR / 2; r++) {
        X[r] = pk2(xv[4 * r], xv[4 * r + 2]);
        Y[r] = pk2(xv[4 * r + 1], xv[4 * r + 3]);
        GX[r] = pk2(0.f, 0.f);
        GY[r] = pk2(0.f, 0.f);
    }
    const float nb = -a.b0 * 1.4426950408889634f;
    const uint64_t A0 = pk2(a.a0, a.a0), B0 = pk2(a.b0, a.b0), NB = pk2(nb, nb);
    const int nw = NW > 0 ? NW : a.nwell;
#pragma unroll
    for (int k = 0; k < nw; k++) {
        const uint64_t MWX = pk2(-a.wc[2 * k], -a.wc[2 * k]), MWY = pk2(-a.wc[2 * k + 1], -a.wc[2 * k + 1]);
#pragma unroll
        for (int r = 0; r < NR / 2; r++) {
            const uint64_t dx = fadd2(X[r], MWX), dy = fadd2(Y[r], MWY);
            const uint64_t u = ffma2(dy, dy, fmul2(dx, dx));
            float t0, t1;
            upk2(fmul2(u, NB), t0, t1);
            const uint64_t eb = pk2(ex2f(t0), ex2f(t1));
            const uint64_t e2 = fmul2(eb, eb), e4 = fmul2(e2, e2), e8 = fmul2(e4, e4);
            const uint64_t ea = fmul2(e8, e2);
            const uint64_t cc = ffma2(B0, eb, fmul2(A0, ea));
            GX[r] = ffma2(cc, dx, GX[r]);
            GY[r] = ffma2(cc, dy, GY[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < NR / 2; r++) {
        upk2(GX[r], gx[2 * r], gx[2 * r + 1]);
        upk2(GY[r], gy[2 * r], gy[2 * r + 1]);
    }
}

// Forces of kGrp columns of one bead (PESK 2: kGrp/2 rings of the 2-D surface;
// PESK 1: kGrp rings of the 1-D quartic).
template <int PESK>
__device__ __forceinline__ void group_forces(const TcArgs &a, const float (&xv)[kGrp], float (&fv)[kGrp]) {
    if constexpr (PESK == 2) {
        constexpr int NR = kGrp / 2;
        float gx[NR], gy[NR];
        if (a.pow10 && a.nwell == 6)  // the mcmod_2dtest default (m = 6)
            grad_2d_pow10_x2<NR, 6>(a, xv, gx, gy);
        else if (a.pow10)
            grad_2d_pow10_x2<NR>(a, xv, gx, gy);
        else
            grad_2d_n<false, NR>(a, xv, gx, gy);
#pragma unroll
        for (int r = 0; r < NR; r++) {
            fv[2 * r] = gx[r];
            fv[2 * r + 1] = gy[r];
        }
    } else {
#pragma unroll
        for (int i = 0; i < kGrp; i++) {
            const float u = xv[i] / a.x0;
            const float w = u * u - 1.0f;
            fv[i] = w * 4.0f * a.H * xv[i] / (a.x0 * a.x0);
        }
    }
}

// Positions x = T q + x* of one group (kGrp columns from c0 of this thread's
// half), read from TMEM; the bead-P values go to the estimator staging.
__device__ __forceinline__ void group_positions(const float *sxa, const float *sxs, uint32_t taddr, int cb, int c0,
                                                int m, bool stage_p, float (&xv)[kGrp], float *xP) {
    __syncwarp();  // tcgen05.ld is .sync.aligned: issue it from a converged warp
    tmem_ldn<kGrp>(taddr + (uint32_t)c0, xv);
    const float fm = (float)(m + 1);
    float xa[kGrp], xs[kGrp];  // 16-byte shared loads (cb + c0 is a multiple of 8)
#pragma unroll
    for (int i = 0; i < kGrp; i += 4) {
        const float4 va = *reinterpret_cast<const float4 *>(&sxa[cb + c0 + i]);
        const float4 vs = *reinterpret_cast<const float4 *>(&sxs[cb + c0 + i]);
        xa[i] = va.x, xa[i + 1] = va.y, xa[i + 2] = va.z, xa[i + 3] = va.w;
        xs[i] = vs.x, xs[i + 1] = vs.y, xs[i + 2] = vs.z, xs[i + 3] = vs.w;
    }
#pragma unroll
    for (int i = 0; i < kGrp; i++) xv[i] += xa[i] + xs[i] * fm;
    if (stage_p && m == kP - 1)
#pragma unroll
        for (int i = 0; i < kGrp; i++) xP[cb + c0 + i] = xv[i];
}

// Estimator of step s-1 (verletmodule.f90:397-403) from the staged bead-P
// positions, one thread per ring of the tile, counted down from the last
// thread (thread 0 issues the GEMMs).
__device__ __forceinline__ void tile_estimator(const TcArgs &a, const float *xP, const double *west, int64_t col0,
                                               int nvalid, int64_t s) {
    const int nd = a.nd, tid = kTileThreads - 1 - (int)threadIdx.x;
    if (tid >= nvalid / nd || (s - 1) < a.imin) return;
    const int64_t ring = col0 / nd + tid;
    double contr = 0.0;
    for (int j = 0; j < nd; j++) contr += west[tid * nd + j] * (-(double)xP[tid * nd + j]);
    RingAcc *r = &a.acc[ring];
    if (r->status == 0) r->dhdr_sum += contr;
    r->nsamples += 1;
}

// This thread's OU normals for its mode m and the 32 columns of its half:
// zc[i] = normal j P + m of the Philox stream of column cb + i at step st.
// Lane e of a quad draws the block of column 4g + e (normals j P + 4 (m/4) ..
// +3, the four modes of the quad), then the quad transposes the 4 x 4 values.
// The quad holds M[e][t] = normal (column 4g + e, mode 4 (m/4) + t) in lane e;
// two exchange stages (lane bit 1, then bit 0) leave M[t][e] in lane e.
__device__ __forceinline__ void quad_transpose(float (&z)[4], int e) {
    const bool b1 = (e & 2) != 0, b0 = (e & 1) != 0;
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const float r = __shfl_xor_sync(0xffffffffu, b1 ? z[j] : z[j + 2], 2);
        const float lo = b1 ? r : z[j], hi = b1 ? z[j + 2] : r;
        z[j] = lo;
        z[j + 2] = hi;
    }
#pragma unroll
    for (int j = 0; j < 4; j += 2) {
        const float r = __shfl_xor_sync(0xffffffffu, b0 ? z[j] : z[j + 1], 1);
        const float lo = b0 ? r : z[j], hi = b0 ? z[j + 1] : r;
        z[j] = lo;
        z[j + 1] = hi;
    }
}

// The 8 OU normals of this thread's mode m for columns cb + c0 .. + 7: lane e
// of a quad draws the blocks of columns cb + c0 + e and cb + c0 + 4 + e.
__device__ __forceinline__ void group_normals(const StepStage *ax, int cb, int c0, int m, uint32_t st,
                                              float (&zg)[kGrp]) {
    const int e = threadIdx.x & 3;
#pragma unroll
    for (int g = 0; g < 2; g++) {
        const int cc = cb + c0 + 4 * g + e;
        const U4 o = philox_block(ax->seed[cc], ax->stream[cc], st, kRngLangevin,
                                  (uint32_t)((ax->jdof[cc] * kP + m) >> 2));
        float z[4];
        box_muller_f(o.x, o.y, z[0], z[1]);
        box_muller_f(o.z, o.w, z[2], z[3]);
        quad_transpose(z, e);
#pragma unroll
        for (int k = 0; k < 4; k++) zg[4 * g + k] = z[k];
    }
}

// Writes the kGrp force values of bead m (one per column c0 + i of this
// thread's half) into the B operand as rows c, K index m.  Adjacent lanes pair
// up with one shuffle per column pair: the even lane stores (m, m+1) of column
// c, the odd lane (m-1, m) of column c+1, 4 bytes each per plane.
// Each lane splits its own values (columns i, i+1 of bead m) into packed hi
// and lo words and swaps them with the partner lane (bead m ^ 1); a byte
// permute then forms the even lane's (m, m+1) word of column i and the odd
// lane's (m-1, m) word of column i+1.  cb + c0 is a multiple of 8.
__device__ __forceinline__ void group_store_operand(unsigned char *Xhi, unsigned char *Xlo, int cb, int c0, int m,
                                                    const float (&fv)[kGrp]) {
    const bool odd = (m & 1) != 0;
    const uint32_t psel = odd ? 0x3276u : 0x5410u;
    const uint32_t off0 = (uint32_t)((cb + c0) >> 3) * kXSbo + (uint32_t)(m >> 3) * kXLbo +
                          (uint32_t)(m & 6) * 2 + (odd ? 16u : 0u);
#pragma unroll
    for (int i = 0; i < kGrp; i += 2) {
        const uint32_t h = pack_bf16(fv[i], fv[i + 1]);
        const uint32_t l = pack_bf16(fv[i] - __uint_as_float(h << 16), fv[i + 1] - __uint_as_float(h & 0xFFFF0000u));
        const uint32_t hp = __shfl_xor_sync(0xffffffffu, h, 1), lp = __shfl_xor_sync(0xffffffffu, l, 1);
        const uint32_t off = off0 + (uint32_t)i * 16;
        *reinterpret_cast<uint32_t *>(Xhi + off) = __byte_perm(h, hp, psel);
        *reinterpret_cast<uint32_t *>(Xlo + off) = __byte_perm(l, lp, psel);
    }
}

// Final pass of an advance: positions x = T q + x* written out, and the
// estimator of the last step.
__global__ void __launch_bounds__(kTileThreads, 2) k_tc_final(TcArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    TcShared *sh = reinterpret_cast<TcShared *>(base + kTileSmemOps);
    StepAux *aux = reinterpret_cast<StepAux *>(base + kTileSmemOps + 256);
    StepStage *sg = &aux->stg[0];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nd = a.nd;
    const int64_t col0 = (int64_t)blockIdx.x * kNc;
    const int nvalid = (int)min((int64_t)kNc, a.nrings * nd - col0);
    const int64_t s = *a.step0 + a.sofs;
    if (tid < kNc) stage_columns(sg, a, col0, nvalid, false);
    const uint32_t tmem = tile_begin(base, sh, a.gT, a.q + col0 * kP, nvalid);
    tile_issue(base, sh, tmem, true);
    const bool ok = tile_wait(sh, 0);
    if (ok) {
        const int m = 32 * (warp & 3) + lane;
        const int cb = 32 * (warp >> 2);
        const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)cb;
#pragma unroll 1
        for (int c0 = 0; c0 < 32; c0 += kGrp) {
            float xv[kGrp];
            group_positions(sg->xa, sg->xs, taddr, cb, c0, m, a.do_est != 0, xv, aux->xP);
            const int nvg = nvalid - cb - c0;
            float *xo = a.x + (size_t)(col0 + cb + c0) * kP + m;
#pragma unroll
            for (int i = 0; i < kGrp; i++)
                if (i < nvg) xo[(size_t)i * kP] = xv[i];
        }
    }
    __syncthreads();  // xP complete
    if (ok && a.do_est) tile_estimator(a, aux->xP, sg->west, col0, nvalid, s);
    tile_release(sh, tmem, a.err, 0);
}

// MD steps sofs .. sofs + nsub - 1 (verletmodule.f90:423-435 in normal-mode
// form) of the rings [r0, r1) of this CTA, r0 = floor(b R / G), r1 =
// floor((b + 1) R / G) for CTA b of G (so every SM gets the same number of
// rings), walked in chunks of up to 64 columns, step after step.  T is copied
// in and TMEM allocated once per launch.  Per chunk and step:
//   GEMM 1: x = T q + x*; estimator of step s-1; forces F(x) split straight
//           into the B operand;
//   GEMM 2: T F; kick, half rotation, OU, half rotation of (q, pi) as one
//           linear map per mode (normals drawn while the state loads), written back.
// The chunk's 8-column groups alternate between the two warp halves (half h
// takes groups h, h + 2, ...), so that a partial chunk loads both halves alike.
// mma_bar completes two phases per chunk (parities 0 and 1).  The per-column
// values of the next chunk are copied in (cp.async) while a chunk runs.
// QT (a CTA holds at most two chunks): q stays in tensor memory for the whole
// launch, TMEM columns 64 (k + 1) .. + 63 for chunk k (lane = mode, as the
// accumulator); it is read from HBM / L2 at the start and written back at the
// end, and only pi goes through global memory every step.
constexpr uint32_t kTmemQt = 256;  // accumulator 64 + two chunks of q, rounded to a power of 2
template <int PESK, bool QT>
__global__ void __launch_bounds__(kTileThreads, 2) k_tc_step(TcArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    unsigned char *Xhi = base + 2 * kOpBytes, *Xlo = Xhi + kXPlane;
    TcShared *sh = reinterpret_cast<TcShared *>(base + kTileSmemOps);
    StepAux *aux = reinterpret_cast<StepAux *>(base + kTileSmemOps + 256);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // The next launch of the advance may begin its set-up now (programmatic
    // dependent launch); it reads no ring state before griddep_wait().
    griddep_launch_dependents();
    const int nd = a.nd;
    const int64_t r0 = (int64_t)blockIdx.x * a.nrings / gridDim.x;
    const int64_t r1 = ((int64_t)blockIdx.x + 1) * a.nrings / gridDim.x;
    const int rpc = kNc / nd;  // rings per chunk
    const int m = 32 * (warp & 3) + lane;  // bead (GEMM 1) / mode (GEMM 2)
    const int hh = warp >> 2;               // warp half: column groups hh, hh + 2, hh + 4, hh + 6
    if (tid < kNc) {  // first chunk's column values, in flight during the set-up
        stage_columns(&aux->stg[0], a, r0 * nd, (int)(min((int64_t)rpc, r1 - r0) * nd), true);
        cp_async_commit();
    }
    const uint32_t tmem = tile_setup(base, sh, a.gT, QT ? kTmemQt : (uint32_t)kNc);
    const uint32_t tlane = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    // kick + rotation + OU + rotation of mode m as one linear map
    const float4 k1 = *reinterpret_cast<const float4 *>(a.fold + (size_t)m * 8);
    const float4 k2 = *reinterpret_cast<const float4 *>(a.fold + (size_t)m * 8 + 4);
    // Set-up above used constant tables only; q, pi, the accumulators and the
    // step counter are read after the previous launch has completed.
    griddep_wait();
    const int64_t s0 = *a.step0 + a.sofs;
    if (QT) {  // q of the CTA's chunks into TMEM (zeros beyond the valid columns)
        int kc = 0;
        for (int64_t rc = r0; rc < r1; rc += rpc, kc++) {
            const int64_t col0 = rc * nd;
            const int nvalid = (int)(min((int64_t)rpc, r1 - rc) * nd);
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const int gc = 16 * g + 8 * hh;
                const float *src = a.q + (size_t)(col0 + gc) * kP + m;
                float v[kGrp];
#pragma unroll
                for (int i = 0; i < kGrp; i++) v[i] = gc + i < nvalid ? src[(size_t)i * kP] : 0.f;
                __syncwarp();
                tmem_st8(tlane + (uint32_t)(64 * (kc + 1) + gc), v);
            }
        }
    }
    uint32_t last_phase = 0;  // parity of the last GEMM issued (for the drain on a timeout)
    bool first = true;
    int buf = 0;
    // Chunks of the CTA's rings, step after step (the rings of a CTA are the
    // same in every step, so no step waits for another CTA).  Three CTA
    // barriers per chunk: operand of GEMM 1 written (tile_load), F operand
    // written, chunk done.  An error (a bounded wait that gave up) ends the
    // loop at the chunk-end barrier.
    int sub = 0;
    for (int64_t rc = r0; sub < a.nsub; buf ^= 1) {
        const uint32_t tq = tlane + (uint32_t)(rc == r0 ? 64 : 128);  // QT: this chunk's q columns
        const int64_t s = s0 + sub;
        const bool est = a.sofs + sub > 0;  // the estimator of step s - 1
        const int64_t col0 = rc * nd;
        const int nvalid = (int)(min((int64_t)rpc, r1 - rc) * nd);
        const StepStage *sg = &aux->stg[buf];
        int64_t rn = rc + rpc;  // the next chunk (the first one of the next step after the last)
        int subn = sub;
        if (rn >= r1) {
            rn = r0;
            subn = sub + 1;
        }
        if (tid < kNc) {  // next chunk's column values into the other buffer
            if (subn < a.nsub)
                stage_columns(&aux->stg[buf ^ 1], a, rn * nd, (int)(min((int64_t)rpc, r1 - rn) * nd), true);
            cp_async_commit();
            cp_async_wait<1>();  // this chunk's copies (made visible by the barrier in tile_load)
        }
        if (QT) {  // the B operand of GEMM 1 from the q columns in TMEM
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const int gc = 16 * g + 8 * hh;
                float v[kGrp];
                __syncwarp();
                tmem_ldn<kGrp>(tq + (uint32_t)gc, v);
                group_store_operand(Xhi, Xlo, gc, 0, m, v);
            }
            fence_async_smem();
            tc_before();
            __syncthreads();
            tc_after();
        } else {
            tile_load(base, a.q + col0 * kP, nvalid);
        }
        tile_issue(base, sh, tmem, first);
        last_phase = 0;
        first = false;
        tile_wait_own(sh, 0);
        {
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const int gc = 16 * g + 8 * hh;  // first column of the group
                if (gc >= nvalid) break;         // warp-uniform
                float xv[kGrp], fv[kGrp];
                group_positions(sg->xa, sg->xs, tlane + (uint32_t)gc, gc, 0, m, est, xv, aux->xP);
                group_forces<PESK>(a, xv, fv);
                group_store_operand(Xhi, Xlo, gc, 0, m, fv);
            }
            fence_async_smem();
        }
        tc_before();
        __syncthreads();  // F operand complete, TMEM reads of GEMM 1 done, xP staged
        tc_after();
        tile_issue(base, sh, tmem, false);
        last_phase = 1;
        if (est) tile_estimator(a, aux->xP, sg->west, col0, nvalid, s);
        tile_wait_own(sh, 1);
        {
            uint32_t badbits = 0;
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const int gc = 16 * g + 8 * hh;
                if (gc < nvalid) {  // warp-uniform
                    const int nvg = nvalid - gc;
                    float *qo = a.q + (size_t)(col0 + gc) * kP + m;
                    float *po = a.pi + (size_t)(col0 + gc) * kP + m;
                    float qv[kGrp], pv[kGrp], gv[kGrp], zg[kGrp];
#pragma unroll
                    for (int i = 0; i < kGrp; i++) {
                        if (!QT) qv[i] = i < nvg ? qo[(size_t)i * kP] : 0.f;
                        pv[i] = i < nvg ? po[(size_t)i * kP] : 0.f;
                    }
                    group_normals(sg, gc, 0, m, (uint32_t)s, zg);  // while the loads are in flight
                    __syncwarp();
                    tmem_ldn<kGrp>(tlane + (uint32_t)gc, gv);
                    if (QT) {
                        __syncwarp();
                        tmem_ldn<kGrp>(tq + (uint32_t)gc, qv);
                    }
                    float qnv[kGrp];
#pragma unroll
                    for (int i = 0; i < kGrp; i++) {
                        const float zk = zg[i];
                        const float pn = fmaf(k1.x, pv[i], fmaf(-k1.w, gv[i], fmaf(k1.y, qv[i], k1.z * zk)));
                        const float qn = fmaf(k2.x, pv[i], fmaf(-k2.w, gv[i], fmaf(k2.y, qv[i], k2.z * zk)));
                        qnv[i] = qn;
                        if (i < nvg) {
                            if (!QT) qo[(size_t)i * kP] = qn;
                            po[(size_t)i * kP] = pn;
                            if (pn != pn) badbits |= 1u << (8 * g + i);
                        }
                    }
                    if (QT) {
                        __syncwarp();
                        tmem_st8(tq + (uint32_t)gc, qnv);
                    }
                }
            }
            badbits = __reduce_or_sync(0xffffffffu, badbits);
            if (lane == 0 && badbits) {
                for (int i = 0; i < 32; i++)
                    if (badbits & (1u << i)) {
                        const int64_t ring = (col0 + 16 * (i >> 3) + 8 * hh + (i & 7)) / nd;
                        if (atomicOr(&a.acc[ring].status, PG_RING_NAN) == 0) a.acc[ring].pad = (int32_t)s;
                    }
            }
        }
        tc_before();
        __syncthreads();  // TMEM and shared memory of this chunk fully read
        tc_after();
        if (sh->err) break;  // CTA-uniform: read after the barrier
        rc = rn;
        sub = subn;
    }
    if (tid < kNc) cp_async_wait<0>();  // no copy left in flight at exit
    if (QT) {  // q back to global memory
        int kc = 0;
        for (int64_t rc = r0; rc < r1; rc += rpc, kc++) {
            const int64_t col0 = rc * nd;
            const int nvalid = (int)(min((int64_t)rpc, r1 - rc) * nd);
#pragma unroll 1
            for (int g = 0; g < 4; g++) {
                const int gc = 16 * g + 8 * hh;
                float v[kGrp];
                __syncwarp();
                tmem_ldn<kGrp>(tlane + (uint32_t)(64 * (kc + 1) + gc), v);
                float *dst = a.q + (size_t)(col0 + gc) * kP + m;
#pragma unroll
                for (int i = 0; i < kGrp; i++)
                    if (gc + i < nvalid) dst[(size_t)i * kP] = v[i];
            }
        }
    }
    tile_release(sh, tmem, a.err, last_phase, QT ? kTmemQt : (uint32_t)kNc);
}

__global__ void k_tc_step_add(int64_t *step, int64_t n) { *step += n; }

// ---------------------------------------------------------------- blocked tensor form (any P <= 512, P % 4 == 0)
// For many-dof surfaces and bead numbers other than 128, an MD step is three
// launches:
//   k_tb_pos:   x = T q + x*                        (blocked split-BF16 GEMM)
//   k_tb_force: F = grad V(x) per (ring, bead), and the estimator of step s-1
//               at bead P (FP32 surface, one thread per ring-bead)
//   k_tb_kick:  T F; kick, half rotation, OU, half rotation of (q, pi)
// T is zero-padded to Pp = 128 mb rows and columns and stored as mb x mb
// blocks of 128 x 128.  A CTA owns 64 state columns (ring-dofs, in any ring
// alignment); its mb accumulators D_i = sum_k T_ik X_k (TMEM columns 64 i ..
// 64 i + 63) are built block by block: per K block k the FP32 rows X_k (zero
// beyond P) are split into the B operand, then for each i the block T_ik is
// bulk-copied in and one 128 x 64 x 128 split-BF16 GEMM is issued and waited for.
constexpr int kMaxMb = 4;

struct TbArgs {
    int64_t nrings;
    int nd, ndim, natom, P, mb;
    float dt;
    int64_t imin;
    const unsigned char *gT;  // mb x mb block image
    const float *coef;        // natom x P x 8: rA rB rC rD ou_a ou_s pscale
    const float *kbase;       // P x 8: the same for a unit mass (k_tb_kick)
    const float4 *kscale;     // natom: (m, sqrt m, 1 / m, 1 / sqrt m) (k_tb_kick)
    const double *mass;
    const double *avec, *bvec, *dbdl;
    const float *Tf;          // P x P FP32 transform (the bead-P row for the Andersen estimator)
    double betan, noutput;
    double dhdr_limit;        // >= 0: re-initialise rings whose estimator exceeds it (Langevin)
    uint8_t *kick;            // per-ring flag: Andersen kick of the current step, or (Langevin) re-initialisation
    const int32_t *ringlam;
    const uint64_t *ringseed;
    const uint32_t *ringstream;
    float *q, *pi, *x, *f;    // [ring][dof][P]
    RingAcc *acc;
    const int64_t *step0;
    int64_t sofs;
    int do_est, do_force;
    int32_t *err;
    PesArgs pes;
};

__device__ __forceinline__ uint32_t tb_tmem_cols(int mb) { return mb == 1 ? 64u : (mb == 2 ? 128u : 256u); }

// Barriers and TMEM for the blocked GEMM; returns the TMEM base.
__device__ __forceinline__ uint32_t tb_begin(TcShared *sh, int mb) {
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&sh->mma_bar, 1);
        mbar_init(&sh->tma_bar, 1);
        mbar_init(&sh->mma_bar2, 1);
        mbar_init(&sh->tma_bar2, 1);
        sh->err = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tmem_alloc(&sh->tmem_slot, tb_tmem_cols(mb));
    }
    tc_before();
    __syncthreads();
    tc_after();
    return sh->tmem_slot;
}

// D_i = sum_k T_ik X_k for the tile whose column c is src[c * P ..].  Thread 0
// drives the blocks j = (k, i) in order, each as two halves: T_hi (copy on
// tma_bar, the 16 T_hi X_hi / T_hi X_lo products committed to mma_bar) and T_lo
// (tma_bar2, the 8 T_lo X_hi products on mma_bar2).  A half's copy for block j
// waits only until the same half of block j - 1 has been read, so copies
// overlap the other half's products, and every mbarrier has at most one phase
// outstanding when it is waited on.  The CTA synchronises once per K block
// (before X is reloaded) and once at the end, after thread 0 has seen the last
// products complete.  Returns whether every wait completed (CTA-uniform).
__device__ __forceinline__ bool tb_gemm(unsigned char *base, TcShared *sh, const TbArgs &a, const float *src,
                                        int nvalid, uint32_t tmem, uint32_t *phase) {
    unsigned char *Xhi = base + 2 * kOpBytes, *Xlo = Xhi + kXPlane;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int P = a.P, mb = a.mb;
    const int c = 8 * warp + (lane & 7);  // operand row written by this thread
    const bool v = c < nvalid;
    const float *row = src + (size_t)(v ? c : 0) * P;
    int j = 0, hi_last = -1, lo_last = -1;  // thread 0: blocks started; last committed halves
    // X_kb: K = beads 128 kb .. 128 kb + 127 of every column (zero beyond P;
    // P % 4 == 0, so each float4 is wholly inside or outside a row); the loads
    // of X_(kb+1) are in flight while the GEMMs of X_kb run
    float4 w[8];
    auto fetch = [&](int kb) {
#pragma unroll
        for (int it = 0; it < 4; it++) {
            const int kg = 128 * kb + 8 * (4 * it + (lane >> 3));
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            w[2 * it] = (v && kg + 4 <= P) ? __ldg(reinterpret_cast<const float4 *>(row + kg)) : z4;
            w[2 * it + 1] = (v && kg + 8 <= P) ? __ldg(reinterpret_cast<const float4 *>(row + kg + 4)) : z4;
        }
    };
    fetch(0);
    for (int kb = 0; kb < mb; kb++) {
#pragma unroll
        for (int it = 0; it < 4; it++) {
            const int kl = 8 * (4 * it + (lane >> 3));
            const float e8[8] = {w[2 * it].x,     w[2 * it].y,     w[2 * it].z,     w[2 * it].w,
                                 w[2 * it + 1].x, w[2 * it + 1].y, w[2 * it + 1].z, w[2 * it + 1].w};
            uint4 hi, lo;
            split8(e8, hi, lo);
            const uint32_t off = x_offset(c, kl);
            *reinterpret_cast<uint4 *>(Xhi + off) = hi;
            *reinterpret_cast<uint4 *>(Xlo + off) = lo;
        }
        fence_async_smem();
        tc_before();
        __syncthreads();  // X_kb written
        tc_after();
        if (kb + 1 < mb) fetch(kb + 1);
        if (tid == 0 && sh->err == 0) {
            const uint32_t th = smem_u32(base), tl = th + kOpBytes, xh = smem_u32(Xhi), xl = smem_u32(Xlo);
            // K-step descriptors as in tile_issue: step 0's plus the byte offset / 16
            const uint64_t dth0 = make_desc(th), dtl0 = make_desc(tl), dxh0 = make_desc_x(xh), dxl0 = make_desc_x(xl);
            for (int ib = 0; ib < mb; ib++, j++) {
                const unsigned char *blk = a.gT + (size_t)(ib * mb + kb) * 2 * kOpBytes;
                const uint32_t d = tmem + (uint32_t)(64 * ib);
                // T_hi half: its buffer is free once the T_hi products of block j - 1 are done
                if (hi_last >= 0 && !mbar_wait(&sh->mma_bar, (uint32_t)hi_last & 1u)) {
                    sh->err |= 2;
                    break;
                }
                mbar_expect_tx(&sh->tma_bar, kOpBytes);
                bulk_g2s(base, blk, 16384, &sh->tma_bar);
                bulk_g2s(base + 16384, blk + 16384, 16384, &sh->tma_bar);
                // T_lo half: free once the T_lo products of block j - 1 are done
                if (lo_last >= 0 && !mbar_wait(&sh->mma_bar2, (uint32_t)lo_last & 1u)) {
                    sh->err |= 2;
                    mbar_wait(&sh->tma_bar, (uint32_t)j & 1u);  // let the T_hi copy land (bounded)
                    break;
                }
                mbar_expect_tx(&sh->tma_bar2, kOpBytes);
                bulk_g2s(base + kOpBytes, blk + kOpBytes, 16384, &sh->tma_bar2);
                bulk_g2s(base + kOpBytes + 16384, blk + kOpBytes + 16384, 16384, &sh->tma_bar2);
                if (!mbar_wait(&sh->tma_bar, (uint32_t)j & 1u)) {
                    sh->err |= 1;
                    mbar_wait(&sh->tma_bar2, (uint32_t)j & 1u);
                    break;
                }
                tc_after();
#pragma unroll
                for (int ks = 0; ks < kP / 16; ks++) {
                    const uint64_t ot = (uint64_t)(ks * 2 * kLBO / 16), ox = (uint64_t)(ks * 2 * kXLbo / 16);
                    mma_bf16_n64(d, dth0 + ot, dxh0 + ox, (kb > 0 || ks > 0) ? 1u : 0u);
                    mma_bf16_n64(d, dth0 + ot, dxl0 + ox, 1u);
                }
                mma_commit(&sh->mma_bar);
                hi_last = j;
                if (!mbar_wait(&sh->tma_bar2, (uint32_t)j & 1u)) {
                    sh->err |= 1;
                    break;
                }
                tc_after();
#pragma unroll
                for (int ks = 0; ks < kP / 16; ks++) {
                    const uint64_t ot = (uint64_t)(ks * 2 * kLBO / 16), ox = (uint64_t)(ks * 2 * kXLbo / 16);
                    mma_bf16_n64(d, dtl0 + ot, dxh0 + ox, 1u);
                }
                mma_commit(&sh->mma_bar2);
                lo_last = j;
            }
            // products still reading X_kb: complete before X is reloaded
            if (kb + 1 < mb && sh->err == 0 && !mbar_wait(&sh->mma_bar2, (uint32_t)lo_last & 1u)) sh->err |= 2;
        }
        if (kb + 1 < mb) {
            tc_before();
            __syncthreads();
            tc_after();
            if (sh->err) break;  // CTA-uniform
        }
    }
    if (tid == 0) {
        // the last products (and any still outstanding after an error) complete
        // before the CTA reads TMEM or releases it; each barrier has at most one
        // phase outstanding here
        if (lo_last >= 0 && !mbar_wait(&sh->mma_bar2, (uint32_t)lo_last & 1u)) sh->err |= 2;
        if (hi_last > lo_last && !mbar_wait(&sh->mma_bar, (uint32_t)hi_last & 1u)) sh->err |= 2;
        tc_before();
    }
    __syncthreads();
    tc_after();
    *phase = 0;  // nothing left for tb_release to drain
    return sh->err == 0;
}

__device__ __forceinline__ void tb_release(TcShared *sh, uint32_t tmem, int mb, int32_t *gerr, uint32_t phase) {
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0 && sh->err) atomicOr(gerr, sh->err);
    if ((sh->err & 2) && phase > 0) mbar_wait(&sh->mma_bar, (phase - 1) & 1u);  // drain (bounded)
    tc_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tmem_dealloc(tmem, tb_tmem_cols(mb));
    }
}

// Positions x = T q + x* of a 64-column tile.
__global__ void __launch_bounds__(kTileThreads, 2) k_tb_pos(TbArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    TcShared *sh = reinterpret_cast<TcShared *>(base + kTileSmemOps);
    TileAux *ax = reinterpret_cast<TileAux *>(base + kTileSmemOps + 256);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nd = a.nd, P = a.P;
    const int64_t col0 = (int64_t)blockIdx.x * kNc;
    const int nvalid = (int)min((int64_t)kNc, a.nrings * nd - col0);
    if (tid == 0) prefetch_l2(a.q + col0 * P, (uint32_t)((size_t)nvalid * P * sizeof(float)));  // the tile's rows
    if (tid < kNc) {
        float xa = 0.f, xs = 0.f;
        if (tid < nvalid) {
            const int64_t ring = (col0 + tid) / nd;
            const int j = (int)(col0 + tid - ring * nd);
            const int lam = a.ringlam[ring];
            xa = (float)a.avec[j];
            xs = (float)((a.bvec[(size_t)lam * nd + j] - a.avec[j]) / (double)(P + 1));
        }
        ax->xa[tid] = xa;
        ax->xs[tid] = xs;
    }
    const uint32_t tmem = tb_begin(sh, a.mb);
    uint32_t phase = 0;
    const bool ok = tb_gemm(base, sh, a, a.q + col0 * P, nvalid, tmem, &phase);
    if (ok) {
        const int cb = 32 * (warp >> 2);
        const int nv = nvalid - cb;
        for (int ib = 0; ib < a.mb; ib++) {
            const int m = 128 * ib + 32 * (warp & 3) + lane;  // bead
            const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(64 * ib + cb);
            const float fm = (float)(m + 1);
#pragma unroll 1
            for (int c0 = 0; c0 < 32; c0 += kGrp) {
                float xv[kGrp];
                __syncwarp();
                tmem_ldn<kGrp>(taddr + (uint32_t)c0, xv);
                float *xo = a.x + (size_t)(col0 + cb + c0) * P + m;
#pragma unroll
                for (int i = 0; i < kGrp; i++)
                    if (m < P && c0 + i < nv) xo[(size_t)i * P] = xv[i] + ax->xa[cb + c0 + i] + ax->xs[cb + c0 + i] * fm;
            }
        }
    }
    tb_release(sh, tmem, a.mb, a.err, phase);
}

// Forces (and the estimator of step s-1 at bead P), one thread per ring-bead.
// The surface indexes a bead's coordinates by atom numbers read from its
// parameter table, so each thread keeps its coordinates and gradient in shared
// memory (row stride nd | 1, odd: conflict-free) and the table is staged there
// too, instead of thread-local arrays and global reads.
constexpr int kForceThreads = 128;
constexpr int kStageParams = 4096;  // parameter tables up to 16 KB are staged in shared memory
__host__ __device__ __forceinline__ int force_stride(int nd) { return nd | 1; }
__host__ __device__ __forceinline__ int staged_params(int nfparams) { return nfparams <= kStageParams ? nfparams : 0; }
static size_t tb_force_smem(int nd, int nfparams) {
    return ((size_t)staged_params(nfparams) * sizeof(float) + 15) / 16 * 16 +
           2 * (size_t)kForceThreads * force_stride(nd) * sizeof(float);
}

__global__ void __launch_bounds__(kForceThreads) k_tb_force(TbArgs a) {
    extern __shared__ __align__(16) unsigned char fsm[];
    const int np = staged_params(a.pes.nparams + pes_fparams_extra(a.pes.id));
    float *sp = reinterpret_cast<float *>(fsm);
    const int ldx = force_stride(a.nd);
    float *sx = reinterpret_cast<float *>(fsm + ((size_t)np * sizeof(float) + 15) / 16 * 16) + threadIdx.x * ldx;
    float *sg = sx + kForceThreads * ldx;
    if (threadIdx.x == 0) {  // the x rows of this block's rings
        const int64_t t0 = (int64_t)blockIdx.x * kForceThreads;
        const int64_t ra = t0 / a.P, rb = min((t0 + kForceThreads - 1) / a.P, a.nrings - 1);
        prefetch_l2(a.x + (size_t)ra * a.nd * a.P, (uint32_t)((size_t)(rb - ra + 1) * a.nd * a.P * sizeof(float)));
    }
    for (int i = threadIdx.x; i < np; i += kForceThreads) sp[i] = a.pes.fparams[i];
    __syncthreads();
    PesArgs pa = a.pes;
    if (np > 0) pa.fparams = sp;  // large tables are read through L1 (uniform addresses)
    const int64_t t = (int64_t)blockIdx.x * kForceThreads + threadIdx.x;
    const int P = a.P, nd = a.nd;
    if (t >= a.nrings * P) return;
    const int64_t ring = t / P;
    const int bead = (int)(t - ring * P);
    const size_t off = (size_t)ring * nd * P + bead;
    for (int j = 0; j < nd; j++) sx[j] = a.x[off + (size_t)j * P];
    if (a.do_force) {
        pes_vgrad<float>(pa, sx, sg);
        for (int j = 0; j < nd; j++) a.f[off + (size_t)j * P] = sg[j];
    }
    const int64_t s = *a.step0 + a.sofs;
    if (a.do_est && bead == P - 1 && (s - 1) >= a.imin) {
        // verletmodule.f90:397-409: an estimate over dHdrlimit is not added; the
        // ring is flagged for re-initialisation (k_ti_reinit, before the kick)
        const int lam = a.ringlam[ring];
        double contr = 0.0;
        for (int j = 0; j < nd; j++)
            contr += a.mass[j / a.ndim] * (-(double)sx[j]) * a.dbdl[(size_t)lam * nd + j];
        RingAcc *r = &a.acc[ring];
        if (a.dhdr_limit < 0.0 || fabs(contr) < a.dhdr_limit) {
            if (r->status == 0) r->dhdr_sum += contr;
        } else if (r->status == 0) {
            r->nreinit += 1;
            a.kick[ring] = 1;
        }
        r->nsamples += 1;
    }
}

// T F, then kick / half rotation / OU / half rotation of a 64-column tile.
__global__ void __launch_bounds__(kTileThreads, 2) k_tb_kick(TbArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    TcShared *sh = reinterpret_cast<TcShared *>(base + kTileSmemOps);
    TileAux *ax = reinterpret_cast<TileAux *>(base + kTileSmemOps + 256);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nd = a.nd, P = a.P;
    const int64_t col0 = (int64_t)blockIdx.x * kNc;
    const int nvalid = (int)min((int64_t)kNc, a.nrings * nd - col0);
    if (tid == 0) {  // the tile's rows of F, q and pi, on their way into L2 while the GEMMs run
        const uint32_t tb = (uint32_t)((size_t)nvalid * P * sizeof(float));
        prefetch_l2(a.f + col0 * P, tb);
        prefetch_l2(a.q + col0 * P, tb);
        prefetch_l2(a.pi + col0 * P, tb);
    }
    const int64_t s = *a.step0 + a.sofs;
    if (tid < kNc) {
        uint64_t sd = 0;
        uint32_t sm = 0;
        const int64_t ring = (col0 + tid) / nd;
        const int j = (int)(col0 + tid - ring * nd);
        if (tid < nvalid) {
            sd = a.ringseed[ring];
            sm = a.ringstream[ring];
        }
        ax->seed[tid] = sd;
        ax->stream[tid] = sm;
        ax->jdof[tid] = j;
        ax->atom[tid] = j / a.ndim;
        ax->msc[tid] = a.kscale[j / a.ndim];
    }
    const uint32_t tmem = tb_begin(sh, a.mb);
    uint32_t phase = 0;
    const bool ok = tb_gemm(base, sh, a, a.f + col0 * P, nvalid, tmem, &phase);
    if (ok) {
        const int cb = 32 * (warp >> 2);
        const int nv = nvalid - cb;
        const int e = lane & 3;
        const float dt = a.dt;
        uint32_t badbits = 0;
        for (int ib = 0; ib < a.mb; ib++) {
            const int m = 128 * ib + 32 * (warp & 3) + lane;  // mode
            const int mc = m < P ? m : P - 1;
            const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(64 * ib + cb);
            // this mode's coefficients for a unit mass; a column's are these times
            // its atom's mass factors (rB m, rC / m, ou_s sqrt m)
            const float4 kb4 = __ldg(reinterpret_cast<const float4 *>(a.kbase + (size_t)mc * 8));
            const float2 kb2 = __ldg(reinterpret_cast<const float2 *>(a.kbase + (size_t)mc * 8 + 4));
#pragma unroll 1
            for (int c0 = 0; c0 < 32; c0 += kGrp) {
                const int nvg = nv - c0;
                float *qo = a.q + (size_t)(col0 + cb + c0) * P + m;
                float *po = a.pi + (size_t)(col0 + cb + c0) * P + m;
                float qv[kGrp], pv[kGrp];
                float4 cfa[kGrp];
                float2 cfb[kGrp];
#pragma unroll
                for (int i = 0; i < kGrp; i++) {  // state first, then the normals
                    const bool in = m < P && i < nvg;
                    qv[i] = in ? qo[(size_t)i * P] : 0.f;
                    pv[i] = in ? po[(size_t)i * P] : 0.f;
                    const float4 ms = ax->msc[cb + c0 + i];
                    cfa[i] = make_float4(kb4.x, kb4.y * ms.x, kb4.z * ms.z, kb4.w);
                    cfb[i] = make_float2(kb2.x, kb2.y * ms.y);
                }
                float gv[kGrp];
                __syncwarp();
                tmem_ldn<kGrp>(taddr + (uint32_t)c0, gv);
#pragma unroll
                for (int g = 0; g < kGrp / 4; g++) {
                    // normals j P + 4 (m / 4) .. + 3 of column c0 + 4g + e, transposed within the quad
                    const int cc = cb + c0 + 4 * g + e;
                    const U4 o = philox_block(ax->seed[cc], ax->stream[cc], (uint32_t)s, kRngLangevin,
                                              (uint32_t)((ax->jdof[cc] * P + m) >> 2));
                    float z[4];
                    box_muller_f(o.x, o.y, z[0], z[1]);
                    box_muller_f(o.z, o.w, z[2], z[3]);
                    quad_transpose(z, e);  // z[k]: this mode's normal for column 4g + k
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const int i = 4 * g + k;
                        if (m < P && i < nvg) {
                            const float4 c4 = cfa[i];
                            const float2 c2 = cfb[i];
                            const float zk = z[k];
                            const float p0 = pv[i] - dt * gv[i];
                            const float q0 = qv[i];
                            float p1 = c4.x * p0 + c4.y * q0;
                            const float q1 = c4.z * p0 + c4.w * q0;
                            p1 = c2.x * p1 + c2.y * zk;
                            const float pn = c4.x * p1 + c4.y * q1;
                            const float qn = c4.z * p1 + c4.w * q1;
                            qo[(size_t)i * P] = qn;
                            po[(size_t)i * P] = pn;
                            if (pn != pn) badbits |= 1u << (c0 + i);
                        }
                    }
                }
            }
        }
        badbits = __reduce_or_sync(0xffffffffu, badbits);
        if (lane == 0 && badbits) {
            for (int i = 0; i < 32; i++)
                if (badbits & (1u << i)) {
                    const int64_t ring = (col0 + cb + i) / nd;
                    if (atomicOr(&a.acc[ring].status, PG_RING_NAN) == 0) a.acc[ring].pad = (int32_t)s;
                }
        }
    }
    tb_release(sh, tmem, a.mb, a.err, phase);
}


// ---------------------------------------------------------------- Andersen thermostat, blocked form
// The Andersen step of time_step_nm (verletmodule.f90:204-234, 291-302):
// resample pi on a Poisson schedule, rotate dt/2, kick with the forces at the
// rotated positions, rotate dt/2; the estimator uses the positions after the
// step (verletmodule.f90:236-245).  Per step: k_tb_and_sched (one thread per
// ring), k_tb_and_pre (resample + first half rotation, one thread per
// element), k_tb_pos, k_tb_force (forces only), k_tb_kick_nm (T F, kick,
// second half rotation), k_tb_and_est (bead-P positions and the estimator).
__global__ void k_tb_and_sched(TbArgs a) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nrings) return;
    const uint32_t st = (uint32_t)(*a.step0 + a.sofs);
    RingAcc *acc = &a.acc[r];
    acc->and_count += 1;
    const bool kick = acc->and_count >= acc->and_rkick;
    if (kick) {
        acc->and_count = 0;
        acc->and_rkick = poisson_d(a.ringseed[r], a.ringstream[r], st, kRngPoisson, a.noutput);
    }
    a.kick[r] = kick ? 1 : 0;
}

__global__ void k_tb_and_pre(TbArgs a) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int P = a.P, nd = a.nd;
    if (e >= a.nrings * nd * P) return;
    const int k = (int)(e % P);
    const int64_t rd = e / P;
    const int dof = (int)(rd % nd);
    const int64_t r = rd / nd;
    const float *cf = a.coef + ((size_t)(dof / a.ndim) * P + k) * 8;
    float pv = a.pi[e], qv = a.q[e];
    if (a.kick[r]) {
        const uint32_t st = (uint32_t)(*a.step0 + a.sofs);
        const double z = normal_d(a.ringseed[r], a.ringstream[r], st, kRngAndersen, (uint32_t)(dof * P + k));
        pv = (float)(z * (double)cf[6]);
    }
    a.pi[e] = cf[0] * pv + cf[1] * qv;
    a.q[e] = cf[2] * pv + cf[3] * qv;
}

// T F, kick, half rotation (no OU): the tile structure of k_tb_kick.
__global__ void __launch_bounds__(kTileThreads, 2) k_tb_kick_nm(TbArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    TcShared *sh = reinterpret_cast<TcShared *>(base + kTileSmemOps);
    TileAux *ax = reinterpret_cast<TileAux *>(base + kTileSmemOps + 256);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nd = a.nd, P = a.P;
    const int64_t col0 = (int64_t)blockIdx.x * kNc;
    const int nvalid = (int)min((int64_t)kNc, a.nrings * nd - col0);
    if (tid == 0) {  // the tile's rows of F, q and pi, on their way into L2 while the GEMMs run
        const uint32_t tb = (uint32_t)((size_t)nvalid * P * sizeof(float));
        prefetch_l2(a.f + col0 * P, tb);
        prefetch_l2(a.q + col0 * P, tb);
        prefetch_l2(a.pi + col0 * P, tb);
    }
    if (tid < kNc) {
        const int64_t ring = (col0 + tid) / nd;
        const int j = (int)(col0 + tid - ring * nd);
        ax->jdof[tid] = j;
        ax->atom[tid] = j / a.ndim;
    }
    const uint32_t tmem = tb_begin(sh, a.mb);
    uint32_t phase = 0;
    const bool ok = tb_gemm(base, sh, a, a.f + col0 * P, nvalid, tmem, &phase);
    if (ok) {
        const int cb = 32 * (warp >> 2);
        const int nv = nvalid - cb;
        const float dt = a.dt;
        uint32_t badbits = 0;
        for (int ib = 0; ib < a.mb; ib++) {
            const int m = 128 * ib + 32 * (warp & 3) + lane;  // mode
            const int mc = m < P ? m : P - 1;
            const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(64 * ib + cb);
#pragma unroll 1
            for (int c0 = 0; c0 < 32; c0 += kGrp) {
                const int nvg = nv - c0;
                float *qo = a.q + (size_t)(col0 + cb + c0) * P + m;
                float *po = a.pi + (size_t)(col0 + cb + c0) * P + m;
                float gv[kGrp];
                __syncwarp();
                tmem_ldn<kGrp>(taddr + (uint32_t)c0, gv);
#pragma unroll
                for (int i = 0; i < kGrp; i++) {
                    if (m < P && i < nvg) {
                        const float *cf = a.coef + ((size_t)ax->atom[cb + c0 + i] * P + mc) * 8;
                        const float4 c4 = __ldg(reinterpret_cast<const float4 *>(cf));
                        const float p0 = po[(size_t)i * P] - dt * gv[i];
                        const float q0 = qo[(size_t)i * P];
                        const float pn = c4.x * p0 + c4.y * q0;
                        const float qn = c4.z * p0 + c4.w * q0;
                        qo[(size_t)i * P] = qn;
                        po[(size_t)i * P] = pn;
                        if (pn != pn) badbits |= 1u << (c0 + i);
                    }
                }
            }
        }
        badbits = __reduce_or_sync(0xffffffffu, badbits);
        if (lane == 0 && badbits) {
            const int64_t s = *a.step0 + a.sofs;
            for (int i = 0; i < 32; i++)
                if (badbits & (1u << i)) {
                    const int64_t ring = (col0 + cb + i) / nd;
                    if (atomicOr(&a.acc[ring].status, PG_RING_NAN) == 0) a.acc[ring].pad = (int32_t)s;
                }
        }
    }
    tb_release(sh, tmem, a.mb, a.err, phase);
}

// Estimator of step s from the positions after the step at bead P:
// x_P = sum_m T[P-1][m] q[m] + x*_P per dof, one warp per ring.
__global__ void k_tb_and_est(TbArgs a) {
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= a.nrings) return;
    const int64_t s = *a.step0 + a.sofs;
    const int P = a.P, nd = a.nd;
    const int lam = a.ringlam[r];
    const float *trow = a.Tf + (size_t)(P - 1) * P;  // T is symmetric: row P-1 = column P-1
    double contr = 0.0;  // summation order of verletmodule.f90:399-403 (dimension outer, atom inner)
    for (int jd = 0; jd < a.ndim; jd++)
        for (int at = 0; at < nd / a.ndim; at++) {
            const int j = at * a.ndim + jd;
            const float *q = a.q + ((size_t)r * nd + j) * P;
            float sum = 0.f;
            for (int m = lane; m < P; m += 32) sum += trow[m] * q[m];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            const double av = a.avec[j], bv = a.bvec[(size_t)lam * nd + j];
            const double xp = (double)sum + av + (bv - av) * (double)P / (double)(P + 1);
            contr += a.mass[at] * (-xp) * a.dbdl[(size_t)lam * nd + j];
        }
    if (lane == 0 && s >= a.imin) {
        RingAcc *acc = &a.acc[r];
        acc->nsamples += 1;
        if (acc->status == 0) acc->dhdr_sum += contr;
    }
}

// Column table of the step kernel (once per batch): column c = ring * nd + j.
__global__ void k_tc_cols(int64_t ncols, int nd, int ndim, int P, const int32_t *ringlam, const uint64_t *ringseed,
                          const uint32_t *ringstream, const double *avec, const double *bvec, const double *dbdl,
                          const double *mass, float *cxa, float *cxs, uint32_t *cstream, int32_t *cjdof,
                          uint64_t *cseed, double *cwest) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    const int64_t ring = c / nd;
    const int j = (int)(c - ring * nd);
    const int lam = ringlam[ring];
    cxa[c] = (float)avec[j];
    cxs[c] = (float)((bvec[(size_t)lam * nd + j] - avec[j]) / (double)(P + 1));
    cstream[c] = ringstream[ring];
    cjdof[c] = j;
    cseed[c] = ringseed[ring];
    cwest[c] = mass[j / ndim] * dbdl[(size_t)lam * nd + j];
}

// ---------------------------------------------------------------- persistent folded step (P = 256)
// One launch runs nsub MD steps of a batch of the 9-atom surface (27 dofs) with
// P = 256, as k_tc_step does for P = 128, with T resident in shared memory.  T
// alone (256 x 256, split-BF16 hi and lo) would take 256 KB; the DST-I symmetry
// T[i][P-1-b] = (-1)^i T[i][b] (0-based) folds it: with u_b = y_b + y_(P-1-b)
// and v_b = y_b - y_(P-1-b), b < 128,
//     (T y)_(2j) = sum_b T[2j][b] u_b,     (T y)_(2j+1) = sum_b T[2j+1][b] v_b,
// so T y is two 128 x 128 products, T_e (even rows) u and T_o (odd rows) v,
// whose images take 128 KB.  One CTA per SM owns an equal range of whole rings,
// cut into chunks of two rings (ring r's dof d at operand row and TMEM column
// 32 r + d); each chunk steps on its own (no grid-wide synchronisation).  Per
// chunk and step:
//   A  positions: the folded operands u and v of q and two GEMMs, T_e u into
//      TMEM columns 0-63 and T_o v into 64-127; TMEM lane j of the first holds
//      bead 2j, of the second bead 2j+1;
//   B  forces: the thread of lane j in warp quarter w % 4 and half h = w / 4
//      reads its bead's 27 dofs (x = T q + x*, the spring line added), forms the
//      estimator of step s - 1 (bead 256) and evaluates the unrolled surface in
//      registers;
//   C  T F: the folded operands of the forces (staged in shared memory) and two
//      GEMMs;
//   D  update: the thread of lane j holds modes 2j and 2j + 1 of 8-column groups
//      (q, pi as float2, coalesced), draws the Langevin normals of both from the
//      two Philox blocks of its quad (pairs exchanged by a quad transpose), and
//      applies the kick / rotation / OU / rotation map per mode.
// The step kernel (k_tf_step, 512 threads) runs two warp groups of 256 on
// alternate chunks of the CTA's range, each with its own 256 TMEM columns
// (positions 0-127, forces 128-255): B and D are long SIMT phases, and the two
// groups run side by side.  B leaves its gradients in the group's force
// columns.  The operand buffer and the force staging in shared memory (the T
// image leaves no room for a second copy) belong to one group at a time: a
// group takes the shared-memory lock to copy its gradients to the staging and
// run C and the A of its next chunk (the positions go to the position
// columns), and releases it before D.
// The read-out pass (k_tf_out, 256 threads) runs A and B only, with the
// positions written out and the estimator of the last step.
constexpr int kFP = 256;                                  // beads
constexpr int kTfThreads = 256;                           // one warp group
constexpr int kTpThreads = 512;                           // the step kernel's two groups
constexpr int kTfStride = kFP + 4;                        // staged force row (floats): rows 4 banks apart
constexpr int kTfCols = 54;                               // staged columns at most
constexpr size_t kTfImg = 4 * (size_t)kOpBytes;           // T_e hi | T_e lo | T_o hi | T_o lo: 128 KB
constexpr int kTfPlane = 64 * kP * 2;                     // one bf16 operand plane, 64 x 128, unpadded: 16 KB
constexpr size_t kTfX = 2 * (size_t)kTfPlane;             // operand hi | lo: 32 KB
constexpr int kTfParams = 1024;                           // surface tables up to 4 KB (staged in shared memory)
constexpr size_t kTfS = (size_t)kTfCols * kTfStride * sizeof(float);

struct TfArgs {
    int64_t nrings;
    int nd, ndim;
    int64_t imin;
    const unsigned char *gT;  // folded image (128 KB)
    const float *fold;        // natom x P x 8 folded kick / rotation / OU map
    const float *mbase;       // P x 8: the map of a unit mass (k_tf_step)
    const float4 *ascale;     // natom: (m, sqrt m, 1 / m, 1 / sqrt m) of each atom (k_tf_step)
    float *q, *pi, *x;        // [ring][dof][P]
    RingAcc *acc;
    const float *cxa, *cxs;
    const uint64_t *cseed;
    const uint32_t *cstream;
    const int32_t *cjdof;
    const double *cwest;
    const int64_t *step0;
    int64_t sofs;
    int nsub, do_est;
    int32_t *err;
    PesArgs pes;
};

struct TpShared {
    uint64_t desc[8];     // operand descriptors: T_e hi, lo, T_o hi, lo, u hi, lo, v hi, lo
    uint64_t mma_bar[2];  // GEMM completion, per warp group (two issuing threads arrive)
    uint64_t tma_bar;     // the image copy
    int32_t err;
    int32_t lock;         // operand buffer and force staging: 0 free, 1 held
    int32_t stop[2];      // a group's exit decision, written by its elected thread
    int32_t go[2];        // a group's issue decision for its current GEMM pair
    uint32_t tmem_slot;
};

// A group's column values of its current chunk (shared memory), loaded at the
// start of each chunk step.
struct TfAux {
    float4 msc[kTfCols];  // the column's atom mass factors (m, sqrt m, 1 / m, 1 / sqrt m)
    float xa[kTfCols], xs[kTfCols];
    double west[kTfCols];
    uint64_t seed[kTfCols];
    uint32_t stream[kTfCols];
    int32_t jdof[kTfCols];
};

static size_t tf_out_smem_bytes() { return 1024 + kTfImg + kTfX + sizeof(TcShared) + 64; }
// 128-byte alignment (the image and operands need 16): the step kernel's layout
// fills the 227 KB a CTA may have.
static size_t tf_step_smem_bytes() {
    return 128 + kTfImg + kTfX + kTfS + 2 * sizeof(TfAux) + kTfParams * sizeof(float) + sizeof(TpShared) + 64;
}

// The group that runs a phase, its barrier and the thread that issues its MMAs:
// the whole CTA, or one 256-thread warp group on named barrier 1 + wg (the
// non-aligned form: the elected thread may arrive after the rest of its warp).
struct CtaSync {
    __device__ __forceinline__ void bar() const { __syncthreads(); }
    __device__ __forceinline__ bool elected() const { return threadIdx.x == 0; }
};
struct WgSync {
    int wg;
    __device__ __forceinline__ void bar() const { asm volatile("barrier.sync %0, 256;" ::"r"(wg + 1) : "memory"); }
    __device__ __forceinline__ bool elected() const { return (threadIdx.x & 255) == 0; }
};
// The error word, which the other group may set at any time.
__device__ __forceinline__ int32_t ld_err(const int32_t *e) { return *reinterpret_cast<const volatile int32_t *>(e); }

// Shared-memory addresses of the image halves and the operand planes.
struct TfOps {
    uint32_t te_hi, te_lo, to_hi, to_lo, xh, xl;
};
// One group's GEMM state: ph counts GEMM slots (the same in every thread of the
// group); nc, in the elected thread, the commits it really issued (after an
// error it issues no more), which the drain at exit waits for.
struct TfGemm {
    uint64_t *mbar, *tbar;
    int32_t *err;
    uint32_t ph, nc;
    bool first;  // the group's first GEMM waits for the image copy
};

// This thread's share of a folded operand: row c = 8 warp + lane % 8 of the 64,
// K chunks kl = 8 (4 it + lane / 8), it = 0..3; u written to the operand now,
// v returned for the second GEMM.  y(k) reads element k of the row (k < 256).
// The operand has the unpadded core-matrix layout of the T image: a warp's
// 16-byte stores cover 512 contiguous bytes, so no padding is needed against
// bank conflicts.
template <typename Ld>
__device__ __forceinline__ void tf_fold_operand(unsigned char *Xhi, unsigned char *Xlo, int c, int lane, bool valid,
                                                Ld ld, float4 (&v)[8]) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int kl = 8 * (4 * it + (lane >> 3));
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 x0 = valid ? ld(kl) : z4, x1 = valid ? ld(kl + 4) : z4;
        const float4 r0 = valid ? ld(kFP - 4 - kl) : z4;  // .w .z .y .x: partners of kl .. kl + 3
        const float4 r1 = valid ? ld(kFP - 8 - kl) : z4;  // partners of kl + 4 .. kl + 7
        const float e8[8] = {x0.x + r0.w, x0.y + r0.z, x0.z + r0.y, x0.w + r0.x,
                             x1.x + r1.w, x1.y + r1.z, x1.z + r1.y, x1.w + r1.x};
        v[2 * it] = make_float4(x0.x - r0.w, x0.y - r0.z, x0.z - r0.y, x0.w - r0.x);
        v[2 * it + 1] = make_float4(x1.x - r1.w, x1.y - r1.z, x1.z - r1.y, x1.w - r1.x);
        uint4 hi, lo;
        split8(e8, hi, lo);
        const uint32_t off = op_offset(c, kl);
        *reinterpret_cast<uint4 *>(Xhi + off) = hi;
        *reinterpret_cast<uint4 *>(Xlo + off) = lo;
    }
}
__device__ __forceinline__ void tf_store_v(unsigned char *Xhi, unsigned char *Xlo, int c, int lane,
                                           const float4 (&v)[8]) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int kl = 8 * (4 * it + (lane >> 3));
        const float e8[8] = {v[2 * it].x, v[2 * it].y, v[2 * it].z, v[2 * it].w,
                             v[2 * it + 1].x, v[2 * it + 1].y, v[2 * it + 1].z, v[2 * it + 1].w};
        uint4 hi, lo;
        split8(e8, hi, lo);
        const uint32_t off = op_offset(c, kl);
        *reinterpret_cast<uint4 *>(Xhi + off) = hi;
        *reinterpret_cast<uint4 *>(Xlo + off) = lo;
    }
}

// Operand complete -> the elected thread issues D = A X (3 split products per K
// step of 16) into TMEM column dcol -> every thread of the group waits for it.
template <class Sync>
__device__ __forceinline__ void tf_gemm(const Sync &sy, TfGemm &g, uint32_t a_hi, uint32_t a_lo, uint32_t xh,
                                        uint32_t xl, uint32_t dtmem) {
    fence_async_smem();
    tc_before();
    sy.bar();
    tc_after();
    if (sy.elected() && ld_err(g.err) == 0) {
        if (g.first && !mbar_wait(g.tbar, 0)) {
            atomicOr(g.err, 1);
        } else {
#pragma unroll
            for (int ks = 0; ks < kP / 16; ks++) {
                const uint64_t dth = make_desc(a_hi + (uint32_t)ks * 2 * kLBO),
                               dtl = make_desc(a_lo + (uint32_t)ks * 2 * kLBO);
                const uint64_t dxh = make_desc(xh + (uint32_t)ks * 2 * kLBO),
                               dxl = make_desc(xl + (uint32_t)ks * 2 * kLBO);
                mma_bf16_n64(dtmem, dth, dxh, ks > 0 ? 1u : 0u);
                mma_bf16_n64(dtmem, dth, dxl, 1u);
                mma_bf16_n64(dtmem, dtl, dxh, 1u);
            }
            mma_commit(g.mbar);
            g.nc++;
        }
    }
    g.first = false;
    sy.bar();  // issued, or an error recorded before any thread of the group waits
    if (ld_err(g.err) == 0 && !mbar_wait(g.mbar, g.ph & 1u)) atomicOr(g.err, 2);
    g.ph++;
    tc_after();
}

// The chunk's operand rows and TMEM columns hold ring r's dof d at 32 r + d
// (kTfRing = 32 per ring, 27 used): ring boundaries fall on 8-column TMEM groups,
// so one rolled loop over the rings (one copy of the surface code) reads and
// writes TMEM at aligned columns.  Column c's index among the chunk's state
// columns (the staging row and the column-value index) is tf_srow(c).
constexpr int kTfRing = 32;
template <int ND>
__device__ __forceinline__ int tf_srow(int c) { return (c / kTfRing) * ND + c % kTfRing; }
template <int ND>
__device__ __forceinline__ bool tf_valid(int c, int nvalid) { return c % kTfRing < ND && tf_srow<ND>(c) < nvalid; }

// A: x = T q of the chunk's state columns [col0, col0 + nvalid) into TMEM
// columns dt (even beads) and dt + 64 (odd beads).
template <int ND, class Sync>
__device__ __forceinline__ void tf_positions(const Sync &sy, TfGemm &g, const TfOps &op, const float *q, int64_t col0,
                                             int nvalid, int c_row, int lane, unsigned char *Xhi, unsigned char *Xlo,
                                             uint32_t dt) {
    float4 v[8];
    const bool valid = tf_valid<ND>(c_row, nvalid);
    const float *row = q + (size_t)(col0 + (valid ? tf_srow<ND>(c_row) : 0)) * kFP;
    tf_fold_operand(Xhi, Xlo, c_row, lane, valid, [&](int k) { return *reinterpret_cast<const float4 *>(row + k); },
                    v);
    tf_gemm(sy, g, op.te_hi, op.te_lo, op.xh, op.xl, dt);
    tf_store_v(Xhi, Xlo, c_row, lane, v);
    tf_gemm(sy, g, op.to_hi, op.to_lo, op.xh, op.xl, dt + 64);
}

// B: the thread's bead b = 2 j + hh of the chunk's rings [rc, rc + RPC): the
// positions from TMEM (tp: the group's position columns at this warp's lane
// quarter) plus the spring line, the estimator of step s - 1 (bead 256), then
// the gradient into TMEM (ts: the group's force columns, free until C; same
// column layout) or, OUT, the positions into x.  The 9-atom surface runs
// unrolled: its coordinates and gradient stay in registers.  Warp-uniform (the
// body issues warp-collective TMEM loads and stores): a wait that gave up in
// another thread may set the error word at any moment.  xa, xs, west: the
// chunk's column values (state column 0 of the chunk first).
template <int ND, int RPC, bool OUT>
__device__ __forceinline__ void tf_beads(const TfArgs &a, const PesArgs &pes, const float *xa, const float *xs,
                                         const double *west, const int32_t *err, uint32_t tp, uint32_t ts, int j,
                                         int hh, int64_t rc, int64_t col0, int nvalid, int64_t s, bool est) {
    static_assert(ND == 27 && RPC * kTfRing <= 64, "k_tf_step evaluates the 9-atom surface, two rings per chunk");
    if (!__all_sync(0xffffffffu, ld_err(err) == 0)) return;
    const int b = 2 * j + hh;
    const float fm = (float)(b + 1);
#pragma unroll 1
    for (int r = 0; r < RPC; r++) {
        if (r * ND >= nvalid) break;  // uniform: whole rings
        const uint32_t cb = (uint32_t)(64 * hh + kTfRing * r);
        float x[ND];
        {
            float t32[kTfRing];
            __syncwarp();
            tmem_ld32(tp + cb, t32);
#pragma unroll
            for (int d = 0; d < ND; d++) x[d] = t32[d];
        }
        const int64_t cr = col0 + r * ND;
        const float *xar = xa + r * ND, *xsr = xs + r * ND;
#pragma unroll
        for (int d = 0; d < ND; d++) x[d] += xar[d] + xsr[d] * fm;
        if (est && b == kFP - 1 && (s - 1) >= a.imin) {  // verletmodule.f90:397-403
            double contr = 0.0;
#pragma unroll
            for (int d = 0; d < ND; d++) contr += west[r * ND + d] * (-(double)x[d]);
            RingAcc *acc = &a.acc[rc + r];
            if (acc->status == 0) acc->dhdr_sum += contr;
            acc->nsamples += 1;
        }
        if (OUT) {
#pragma unroll
            for (int d = 0; d < ND; d++) a.x[(size_t)(cr + d) * kFP + b] = x[d];
        } else {
            float g[ND];
            pes_synth9_canon<float>(pes, x, g);
            float t32[kTfRing];
#pragma unroll
            for (int d = 0; d < kTfRing; d++) t32[d] = d < ND ? g[d] : 0.f;
            __syncwarp();
            tmem_st32(ts + cb, t32);
        }
    }
}

// The staged gradients (TMEM, as tf_beads left them) into the force staging in
// shared memory, row r ND + d, bead b; warp-uniform, as B.
template <int ND, int RPC>
__device__ __forceinline__ void tf_stage_copy(const int32_t *err, uint32_t ts, int j, int hh, int nvalid, float *S) {
    if (!__all_sync(0xffffffffu, ld_err(err) == 0)) return;
    const int b = 2 * j + hh;
#pragma unroll
    for (int r = 0; r < RPC; r++) {
        if (r * ND >= nvalid) break;
        float t32[kTfRing];
        __syncwarp();
        tmem_ld32(ts + (uint32_t)(64 * hh + kTfRing * r), t32);
#pragma unroll
        for (int d = 0; d < ND; d++) S[(r * ND + d) * kTfStride + b] = t32[d];
    }
}

// D: kick, half rotation, OU, half rotation of modes 2j and 2j + 1 of the
// chunk's columns, the forces in modes read from TMEM (tf: the group's force
// columns at this warp's lane quarter), 8-column groups in two halves of 4 (a
// half lies in one ring).  Written for two 27-dof rings per chunk.  The map of
// (atom, mode) is the unit-mass map of the mode times the atom's mass factors:
// the bead masses m (lambda_k tau)^2 make the mode frequencies 1 / tau and the
// OU factor exp(-gamma dt / tau) mass-free, so [K11 K12 N1 D1 | K21 K22 N2 D2]
// scale as [1, m, sqrt m, 1 | 1 / m, 1, 1 / sqrt m, 1 / m] (checked on the host
// against the per-atom maps).  Each half first issues its q and pi loads, then
// draws the normals while they are in flight.  Warp-uniform, as B.
template <int ND>
__device__ __forceinline__ void tf_update(const TfArgs &a, const TfAux &ax, const int32_t *err, uint32_t tf, int j,
                                          int hh, int lane, int64_t col0, int nvalid, int64_t s) {
    if (!__all_sync(0xffffffffu, ld_err(err) == 0)) return;
    const int e = lane & 3;
    const int mq = 2 * (j - e);  // the quad's modes mq .. mq + 7
    // unit-mass maps of modes 2j and 2j + 1
    const float4 b1e = __ldg(reinterpret_cast<const float4 *>(a.mbase + (size_t)(2 * j) * 8));
    const float4 b2e = __ldg(reinterpret_cast<const float4 *>(a.mbase + (size_t)(2 * j) * 8 + 4));
    const float4 b1o = __ldg(reinterpret_cast<const float4 *>(a.mbase + (size_t)(2 * j + 1) * 8));
    const float4 b2o = __ldg(reinterpret_cast<const float4 *>(a.mbase + (size_t)(2 * j + 1) * 8 + 4));
#pragma unroll 1
    for (int g = 0; g < 4; g++) {
        // the 8 column groups of two rings (3 full and one with 3 dofs each) split
        // 27 + 27: half 0 takes groups 0, 1, 2, 7, half 1 groups 3, 4, 5, 6
        const int gc = 8 * (hh == 0 ? (g < 3 ? g : 7) : 3 + g);
        if (!tf_valid<ND>(gc, nvalid)) continue;  // warp-uniform; the group's first column decides
        float gE[8], gO[8];
        __syncwarp();
        tmem_ld8x2(tf + (uint32_t)gc, tf + (uint32_t)(64 + gc), gE, gO);
#pragma unroll
        for (int t4 = 0; t4 < 8; t4 += 4) {
            const int d0 = (gc + t4) % kTfRing;
            if (d0 >= ND) break;  // warp-uniform: the ring's padding
            const int sc0 = tf_srow<ND>(gc + t4);  // state column of the half's first column
            const int nt = min(4, ND - d0);
            float2 q2[4], p2[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int col = sc0 + (t < nt ? t : 0);
                q2[t] = *reinterpret_cast<const float2 *>(a.q + (size_t)(col0 + col) * kFP + 2 * j);
                p2[t] = *reinterpret_cast<const float2 *>(a.pi + (size_t)(col0 + col) * kFP + 2 * j);
            }
            float zE[4], zO[4];
            {
                const bool ok = e < nt;  // this lane draws the blocks of state column sc0 + e
                const int32_t jd = ok ? ax.jdof[sc0 + e] : 0;
                const uint64_t sd = ok ? ax.seed[sc0 + e] : 0;
                const uint32_t sm = ok ? ax.stream[sc0 + e] : 0;
                const uint32_t blk = (uint32_t)((jd * kFP + mq) >> 2);
                const U4 oa = philox_block(sd, sm, (uint32_t)s, kRngLangevin, blk);
                const U4 ob = philox_block(sd, sm, (uint32_t)s, kRngLangevin, blk + 1);
                box_muller_f(oa.x, oa.y, zE[0], zO[0]);  // modes mq, mq + 1
                box_muller_f(oa.z, oa.w, zE[1], zO[1]);  // mq + 2, mq + 3
                box_muller_f(ob.x, ob.y, zE[2], zO[2]);
                box_muller_f(ob.z, ob.w, zE[3], zO[3]);
                quad_transpose(zE, e);  // zE[t]: mode 2j of state column sc0 + t
                quad_transpose(zO, e);  // zO[t]: mode 2j + 1
            }
#pragma unroll
            for (int t = 0; t < 4; t++) {
                if (t >= nt) break;
                const int col = sc0 + t;
                const float4 ms = ax.msc[col];  // m, sqrt m, 1 / m, 1 / sqrt m
                const float ge = gE[t4 + t], go = gO[t4 + t];
                float2 pn, qn;
                pn.x = fmaf(b1e.x, p2[t].x, fmaf(-b1e.w, ge, fmaf(b1e.y * ms.x, q2[t].x, (b1e.z * ms.y) * zE[t])));
                qn.x = fmaf(b2e.x * ms.z, p2[t].x,
                            fmaf(-(b2e.w * ms.z), ge, fmaf(b2e.y, q2[t].x, (b2e.z * ms.w) * zE[t])));
                pn.y = fmaf(b1o.x, p2[t].y, fmaf(-b1o.w, go, fmaf(b1o.y * ms.x, q2[t].y, (b1o.z * ms.y) * zO[t])));
                qn.y = fmaf(b2o.x * ms.z, p2[t].y,
                            fmaf(-(b2o.w * ms.z), go, fmaf(b2o.y, q2[t].y, (b2o.z * ms.w) * zO[t])));
                *reinterpret_cast<float2 *>(a.q + (size_t)(col0 + col) * kFP + 2 * j) = qn;
                *reinterpret_cast<float2 *>(a.pi + (size_t)(col0 + col) * kFP + 2 * j) = pn;
                if (pn.x != pn.x || pn.y != pn.y) {
                    const int64_t ring = (col0 + col) / ND;
                    if (atomicOr(&a.acc[ring].status, PG_RING_NAN) == 0) a.acc[ring].pad = (int32_t)s;
                }
            }
        }
    }
}

// Step kernel, operands in pairs: u in X, v in the staging region (free once
// the fold of the staged forces has read it), so that the two GEMMs of a
// transform are issued back to back under one commit.
struct TfPair {
    unsigned char *uhi, *ulo, *vhi, *vlo;
    uint32_t su_hi, su_lo, sv_hi, sv_lo;  // shared-space addresses of the same
};
// This thread's 16 loads of a folded operand row (x0, x1, r0, r1 per K quarter,
// as tf_fold_operand reads them), issued together.
template <typename Ld>
__device__ __forceinline__ void tf_fold_load(float4 (&L)[16], int lane, bool valid, Ld ld) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int kl = 8 * (4 * it + (lane >> 3));
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        L[4 * it] = valid ? ld(kl) : z4;
        L[4 * it + 1] = valid ? ld(kl + 4) : z4;
        L[4 * it + 2] = valid ? ld(kFP - 4 - kl) : z4;
        L[4 * it + 3] = valid ? ld(kFP - 8 - kl) : z4;
    }
}
// u and v of the loaded row into both operands of the pair.
__device__ __forceinline__ void tf_fold_store(const float4 (&L)[16], const TfPair &x, int c, int lane) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
        const int kl = 8 * (4 * it + (lane >> 3));
        const float4 x0 = L[4 * it], x1 = L[4 * it + 1], r0 = L[4 * it + 2], r1 = L[4 * it + 3];
        const float e8[8] = {x0.x + r0.w, x0.y + r0.z, x0.z + r0.y, x0.w + r0.x,
                             x1.x + r1.w, x1.y + r1.z, x1.z + r1.y, x1.w + r1.x};
        const float o8[8] = {x0.x - r0.w, x0.y - r0.z, x0.z - r0.y, x0.w - r0.x,
                             x1.x - r1.w, x1.y - r1.z, x1.z - r1.y, x1.w - r1.x};
        const uint32_t off = op_offset(c, kl);
        uint4 hi, lo;
        split8(e8, hi, lo);
        *reinterpret_cast<uint4 *>(x.uhi + off) = hi;
        *reinterpret_cast<uint4 *>(x.ulo + off) = lo;
        split8(o8, hi, lo);
        *reinterpret_cast<uint4 *>(x.vhi + off) = hi;
        *reinterpret_cast<uint4 *>(x.vlo + off) = lo;
    }
}
// Both operands complete -> T_e u into TMEM column dt, issued by the group's
// thread 0, and T_o v into dt + 64, issued by its thread 32, each under its own
// commit (the group's barrier counts two arrivals).  The descriptors of K step
// ks are the base ones (TpShared::desc) plus 16 ks: 256 bytes of start address.
// The elected thread decides for both whether the pair is issued.  The group
// waits with tf_gemm_wait.
__device__ __forceinline__ void tf_gemm_pair_issue(const WgSync &sy, TfGemm &g, TpShared *sh, uint32_t dt) {
    fence_async_smem();
    tc_before();
    const int wg = sy.wg, wt = threadIdx.x & 255;
    if (wt == 0) {
        int go = ld_err(g.err) == 0;
        if (go && g.first && !mbar_wait(g.tbar, 0)) {
            atomicOr(g.err, 1);
            go = 0;
        }
        sh->go[wg] = go;
    }
    sy.bar();
    tc_after();
    if ((wt == 0 || wt == 32) && sh->go[wg]) {
        const int h = wt >> 5;  // 0: T_e u, 1: T_o v
        const uint64_t ah = sh->desc[2 * h], al = sh->desc[2 * h + 1];
        const uint64_t xh = sh->desc[4 + 2 * h], xl = sh->desc[5 + 2 * h];
        const uint32_t d = dt + 64u * (uint32_t)h;
#pragma unroll
        for (int ks = 0; ks < kP / 16; ks++) {
            const uint64_t o = 16ull * (uint64_t)ks;
            mma_bf16_n64(d, ah + o, xh + o, ks > 0 ? 1u : 0u);
            mma_bf16_n64(d, ah + o, xl + o, 1u);
            mma_bf16_n64(d, al + o, xh + o, 1u);
        }
        mma_commit(g.mbar);
        g.nc++;
    }
    g.first = false;
    sy.bar();  // issued, or not, before any thread of the group waits
}
__device__ __forceinline__ void tf_gemm_wait(TfGemm &g) {
    if (ld_err(g.err) == 0 && !mbar_wait(g.mbar, g.ph & 1u)) atomicOr(g.err, 2);
    g.ph++;
    tc_after();
}
// A of the step kernel (the group holds the lock): q of the chunk's state
// columns [col0, col0 + nvalid) into TMEM columns dt (even beads), dt + 64.
template <int ND>
__device__ __forceinline__ void tf_positions_pair(const WgSync &sy, TfGemm &g, TpShared *sh, const TfPair &x,
                                                  const float *q, int64_t col0, int nvalid, int c_row, int lane,
                                                  uint32_t dt) {
    float4 L[16];
    const bool valid = tf_valid<ND>(c_row, nvalid);
    const float *row = q + (size_t)(col0 + (valid ? tf_srow<ND>(c_row) : 0)) * kFP;
    tf_fold_load(L, lane, valid, [&](int k) { return *reinterpret_cast<const float4 *>(row + k); });
    tf_fold_store(L, x, c_row, lane);
    tf_gemm_pair_issue(sy, g, sh, dt);
    tf_gemm_wait(g);
}
// C of the step kernel (the group holds the lock), then, when next, the A of
// the group's next chunk: T F of the staged forces into TMEM columns df, df +
// 64; the next chunk's q rows are loaded while those GEMMs run, then its
// positions go to dp, dp + 64.  next is uniform over the group.
template <int ND>
__device__ __forceinline__ void tf_modes_then_positions(const WgSync &sy, TfGemm &g, TpShared *sh, const TfPair &x,
                                                        const float *S, int nvalid, uint32_t df, bool next,
                                                        const float *q, int64_t ncol0, int nnvalid, int c_row,
                                                        int lane, uint32_t dp) {
    {
        float4 v[8];
        const bool valid = tf_valid<ND>(c_row, nvalid);
        const float *row = S + (size_t)(valid ? tf_srow<ND>(c_row) : 0) * kTfStride;
        tc_before();
        sy.bar();  // staged forces complete
        tc_after();
        tf_fold_operand(x.uhi, x.ulo, c_row, lane, valid,
                        [&](int k) { return *reinterpret_cast<const float4 *>(row + k); }, v);
        sy.bar();  // every thread has read the staging, which now takes v
        tf_store_v(x.vhi, x.vlo, c_row, lane, v);
    }
    tf_gemm_pair_issue(sy, g, sh, df);
    if (next) {
        float4 L[16];
        const bool valid = tf_valid<ND>(c_row, nnvalid);
        const float *row = q + (size_t)(ncol0 + (valid ? tf_srow<ND>(c_row) : 0)) * kFP;
        tf_fold_load(L, lane, valid, [&](int k) { return *reinterpret_cast<const float4 *>(row + k); });
        tf_gemm_wait(g);  // the operands are read: they take the next chunk's q
        tf_fold_store(L, x, c_row, lane);
        tf_gemm_pair_issue(sy, g, sh, dp);
    }
    tf_gemm_wait(g);
}

// The shared-memory lock: the group's elected thread takes it (bounded spin;
// on giving up it records an error and the group goes on without it, issuing
// no further MMAs), then the group's barrier.
__device__ __forceinline__ bool tf_lock(const WgSync &sy, TpShared *sh) {
    bool held = false;
    if (sy.elected()) {
        const uint64_t t0 = globaltimer_ns();
        for (long long i = 0; i < kSpinLimit; i++) {
            if (atomicCAS(&sh->lock, 0, 1) == 0) {
                held = true;
                break;
            }
            if ((i & 63) == 63 && globaltimer_ns() - t0 > kWaitLimitNs) break;
            __nanosleep(64);
        }
        __threadfence_block();
        if (!held) atomicOr(&sh->err, 8);
    }
    tc_before();
    sy.bar();
    tc_after();
    return held;
}
// Every thread of the group is done with the operand and the staging (its GEMMs
// completed), then the elected thread releases the lock it holds.
__device__ __forceinline__ void tf_unlock(const WgSync &sy, TpShared *sh, bool held) {
    tc_before();
    sy.bar();
    tc_after();
    if (sy.elected() && held) {
        __threadfence_block();
        atomicExch(&sh->lock, 0);
    }
}

template <int ND, int RPC>
__global__ void __launch_bounds__(kTpThreads, 1) k_tf_step(TfArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(dsm) + 127) & ~(uintptr_t)127);
    unsigned char *Xhi = base + kTfImg, *Xlo = Xhi + kTfPlane;
    float *S = reinterpret_cast<float *>(base + kTfImg + kTfX);
    TfAux *auxes = reinterpret_cast<TfAux *>(base + kTfImg + kTfX + kTfS);
    float *par = reinterpret_cast<float *>(base + kTfImg + kTfX + kTfS + 2 * sizeof(TfAux));
    TpShared *sh = reinterpret_cast<TpShared *>(base + kTfImg + kTfX + kTfS + 2 * sizeof(TfAux) +
                                                kTfParams * sizeof(float));
    const int tid = threadIdx.x, wg = tid >> 8, wtid = tid & 255, wwarp = wtid >> 5, lane = tid & 31;
    TfAux &ax = auxes[tid >> 8];
    const WgSync sy{wg};
    const TfOps op{smem_u32(base), smem_u32(base) + kOpBytes, smem_u32(base) + 2 * kOpBytes,
                   smem_u32(base) + 3 * kOpBytes, smem_u32(Xhi), smem_u32(Xlo)};
    if (tid == 0) {
        mbar_init(&sh->mma_bar[0], 2);
        mbar_init(&sh->mma_bar[1], 2);
        mbar_init(&sh->tma_bar, 1);
        sh->err = 0;
        sh->lock = 0;
        sh->stop[0] = sh->stop[1] = 0;
        const uint32_t sv = smem_u32(S);
        const uint32_t ad[8] = {op.te_hi, op.te_lo, op.to_hi, op.to_lo, op.xh, op.xl, sv, sv + (uint32_t)kTfPlane};
        for (int i = 0; i < 8; i++) sh->desc[i] = make_desc(ad[i]);
        fence_barrier_init();
    }
    // the surface table (uniform reads in every evaluation: L1 is what shared
    // memory leaves, so it is staged); the host checks that it fits
    const int np = a.pes.nparams + pes_fparams_extra(a.pes.id);
    for (int i = tid; i < np; i += kTpThreads) par[i] = a.pes.fparams[i];
    __syncthreads();
    if (tid == 0) {  // the folded image, 128 KB, once per launch
        mbar_expect_tx(&sh->tma_bar, (uint32_t)kTfImg);
#pragma unroll 1
        for (int i = 0; i < (int)(kTfImg / 16384); i++) bulk_g2s(base + i * 16384, a.gT + i * 16384, 16384, &sh->tma_bar);
    }
    if (tid < 32) {
        __syncwarp();
        tmem_alloc(&sh->tmem_slot, 512);
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tcol = sh->tmem_slot + 256u * (uint32_t)wg;  // positions: +0, forces: +128
    const uint32_t tq = tcol + ((uint32_t)(32 * (wwarp & 3)) << 16);
    const int j = 32 * (wwarp & 3) + lane;  // TMEM lane
    const int hh = wwarp >> 2;              // half: even / odd beads (B), column groups (D)
    const int c_row = 8 * wwarp + (lane & 7);
    TfGemm G{&sh->mma_bar[wg], &sh->tma_bar, &sh->err, 0, 0, true};
    PesArgs pes = a.pes;
    pes.fparams = par;
    const int64_t r0 = (int64_t)blockIdx.x * a.nrings / gridDim.x;
    const int64_t r1 = ((int64_t)blockIdx.x + 1) * a.nrings / gridDim.x;
    const int64_t s0 = *a.step0 + a.sofs;
    // this group's chunks: wg, wg + 2, ... of the range's nch; item k is chunk
    // k % nown at sub-step k / nown
    const int64_t nch = (r1 - r0 + RPC - 1) / RPC;
    const int64_t nown = nch > wg ? (nch - wg + 1) / 2 : 0;
    const int64_t K = nown * a.nsub;
    auto ring_of = [&](int64_t k) { return r0 + (int64_t)RPC * (wg + 2 * (k % nown)); };
    auto nvalid_of = [&](int64_t rc) { return (int)(min((int64_t)RPC, r1 - rc) * ND); };
    const TfPair xp{Xhi, Xlo, reinterpret_cast<unsigned char *>(S), reinterpret_cast<unsigned char *>(S) + kTfPlane,
                    op.xh, op.xl, smem_u32(S), smem_u32(S) + kTfPlane};
    if (K > 0) {
        const bool held = tf_lock(sy, sh);
        const int64_t rc = ring_of(0);
        tf_positions_pair<ND>(sy, G, sh, xp, a.q, rc * ND, nvalid_of(rc), c_row, lane, tcol);
        tf_unlock(sy, sh, held);
    }
#pragma unroll 1
    for (int64_t k = 0; k < K; k++) {
        const int64_t sub = k / nown, rc = ring_of(k), col0 = rc * ND;
        const int nvalid = nvalid_of(rc);
        const int64_t s = s0 + sub;
        if (wtid < kTfCols) {  // the chunk's column values (the group's D of the last chunk has read them)
            const bool ok = wtid < nvalid;
            const int64_t c = col0 + wtid;
            ax.xa[wtid] = ok ? a.cxa[c] : 0.f;
            ax.xs[wtid] = ok ? a.cxs[c] : 0.f;
            ax.west[wtid] = ok ? a.cwest[c] : 0.0;
            ax.seed[wtid] = ok ? a.cseed[c] : 0;
            ax.stream[wtid] = ok ? a.cstream[c] : 0;
            ax.jdof[wtid] = ok ? a.cjdof[c] : 0;
            ax.msc[wtid] = ok ? a.ascale[a.cjdof[c] / a.ndim] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (sy.elected()) {  // into L2 while the forces run: this chunk's state for D, the next chunk's q for A
            prefetch_l2(a.pi + (size_t)col0 * kFP, (uint32_t)(nvalid * kFP * sizeof(float)));
            prefetch_l2(a.q + (size_t)col0 * kFP, (uint32_t)(nvalid * kFP * sizeof(float)));
            if (k + 1 < K) {
                const int64_t rn = ring_of(k + 1);
                prefetch_l2(a.q + (size_t)rn * ND * kFP, (uint32_t)(nvalid_of(rn) * kFP * sizeof(float)));
            }
        }
        sy.bar();
        tf_beads<ND, RPC, false>(a, pes, ax.xa, ax.xs, ax.west, &sh->err, tq, tq + 128, j, hh, rc, col0, nvalid, s,
                                 a.sofs + sub > 0);
        const bool held = tf_lock(sy, sh);
        tf_stage_copy<ND, RPC>(&sh->err, tq + 128, j, hh, nvalid, S);
        {
            // the next chunk's positions (its q is final: it stepped before this one)
            const bool next = nown >= 2 && k + 1 < K;
            const int64_t rn = next ? ring_of(k + 1) : rc;
            tf_modes_then_positions<ND>(sy, G, sh, xp, S, nvalid, tcol + 128, next, a.q, rn * ND, nvalid_of(rn),
                                        c_row, lane, tcol);
        }
        tf_unlock(sy, sh, held);
        tf_update<ND>(a, ax, &sh->err, tq + 128, j, hh, lane, col0, nvalid, s);
        if (nown == 1 && k + 1 < K) {  // one chunk: its next positions need this update
            const bool h2 = tf_lock(sy, sh);
            tf_positions_pair<ND>(sy, G, sh, xp, a.q, col0, nvalid, c_row, lane, tcol);
            tf_unlock(sy, sh, h2);
        }
        sy.bar();
        if (sy.elected()) sh->stop[wg] = ld_err(&sh->err);
        sy.bar();
        if (sh->stop[wg]) break;  // group-uniform: written before the barrier, rewritten only after the next
    }
    // let whatever is in flight land (immediate when it has), then release TMEM:
    // the group's last committed GEMM (after a failed wait it may still run) and
    // the image copy (outstanding if no GEMM waited for it); both waits bounded
    if ((wtid == 0 || wtid == 32) && G.nc > 0) mbar_wait(G.mbar, (G.nc - 1) & 1u);
    tc_before();
    __syncthreads();
    if (tid == 0) {
        mbar_wait(&sh->tma_bar, 0);
        if (sh->err) atomicOr(a.err, sh->err);
    }
    __syncthreads();
    if (tid < 32) {
        __syncwarp();
        tc_after();
        tmem_dealloc(sh->tmem_slot, 512);
    }
}

// Read-out pass: A and B of every chunk, positions written out, the estimator
// of the last step when do_est.
template <int ND, int RPC>
__global__ void __launch_bounds__(kTfThreads, 1) k_tf_out(TfArgs a) {
    extern __shared__ unsigned char dsm[];
    unsigned char *base = align1k(dsm);
    unsigned char *Xhi = base + kTfImg, *Xlo = Xhi + kTfPlane;
    TcShared *sh = reinterpret_cast<TcShared *>(base + kTfImg + kTfX);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const CtaSync sy;
    const TfOps op{smem_u32(base), smem_u32(base) + kOpBytes, smem_u32(base) + 2 * kOpBytes,
                   smem_u32(base) + 3 * kOpBytes, smem_u32(Xhi), smem_u32(Xlo)};
    if (tid == 0) {
        mbar_init(&sh->mma_bar, 1);
        mbar_init(&sh->tma_bar, 1);
        sh->err = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_expect_tx(&sh->tma_bar, (uint32_t)kTfImg);
#pragma unroll 1
        for (int i = 0; i < (int)(kTfImg / 16384); i++) bulk_g2s(base + i * 16384, a.gT + i * 16384, 16384, &sh->tma_bar);
    }
    if (warp == 0) {
        __syncwarp();
        tmem_alloc(&sh->tmem_slot, 128);
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = sh->tmem_slot;
    const uint32_t tq = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    const int j = 32 * (warp & 3) + lane;
    const int hh = warp >> 2;
    const int c_row = 8 * warp + (lane & 7);
    TfGemm G{&sh->mma_bar, &sh->tma_bar, &sh->err, 0, 0, true};
    const int64_t r0 = (int64_t)blockIdx.x * a.nrings / gridDim.x;
    const int64_t r1 = ((int64_t)blockIdx.x + 1) * a.nrings / gridDim.x;
    const int64_t s = *a.step0 + a.sofs;
#pragma unroll 1
    for (int64_t rc = r0; rc < r1; rc += RPC) {
        const int64_t col0 = rc * ND;
        const int nvalid = (int)(min((int64_t)RPC, r1 - rc) * ND);
        tf_positions<ND>(sy, G, op, a.q, col0, nvalid, c_row, lane, Xhi, Xlo, tmem);
        tf_beads<ND, RPC, true>(a, a.pes, a.cxa + col0, a.cxs + col0, a.cwest + col0, &sh->err, tq, 0, j, hh, rc,
                                col0, nvalid, s, a.do_est != 0);
        tc_before();
        __syncthreads();  // TMEM and operand of this chunk fully read
        tc_after();
        if (sh->err) break;  // CTA-uniform: read after the barrier
    }
    if (tid == 0) {
        if (sh->err) atomicOr(a.err, sh->err);
        if (G.nc > 0) mbar_wait(&sh->mma_bar, (G.nc - 1) & 1u);
        mbar_wait(&sh->tma_bar, 0);
    }
    tc_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        tc_after();
        tmem_dealloc(tmem, 128);
    }
}

// Host: split-BF16 image of T, zero-padded to mb x mb blocks of 128 x 128
// (mb = ceil(P / 128)); block (ib, kb) is a 64 KB [hi | lo] pair in the K-major
// core-matrix layout of the A operand, at (ib mb + kb) 64 KB.
static int blocks_for(int P) { return (P + kP - 1) / kP; }

static void build_split_image(int P, std::vector<unsigned char> &img) {
    std::vector<double> T;
    build_transmatrix(P, T);
    const int mb = blocks_for(P);
    img.assign((size_t)mb * mb * 2 * kOpBytes, 0);
    for (int n = 0; n < P; n++)
        for (int k = 0; k < P; k++) {
            double v = T[(size_t)n + (size_t)P * k];
            __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
            double r = v - (double)__bfloat162float(hi);
            __nv_bfloat16 lo = __float2bfloat16_rn((float)r);
            const size_t blk = ((size_t)(n / kP) * mb + (size_t)(k / kP)) * 2 * kOpBytes;
            const uint32_t off = op_offset(n % kP, k % kP);
            memcpy(&img[blk + off], &hi, 2);
            memcpy(&img[blk + kOpBytes + off], &lo, 2);
        }
}

// The folded image of T for P = 256 (k_tf_step): [T_e hi | T_e lo | T_o hi |
// T_o lo], T_e[r][c] = T[2r][c] and T_o[r][c] = T[2r+1][c] for r, c < 128, each a
// 128 x 128 K-major core-matrix image laid out as the P = 128 one.
static void build_fold_image(std::vector<unsigned char> &img) {
    std::vector<double> T;
    build_transmatrix(kFP, T);
    img.assign(kTfImg, 0);
    for (int h = 0; h < 2; h++)
        for (int r = 0; r < kFP / 2; r++)
            for (int c = 0; c < kFP / 2; c++) {
                const double v = T[(size_t)(2 * r + h) + (size_t)kFP * c];
                __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
                const double rem = v - (double)__bfloat162float(hi);
                __nv_bfloat16 lo = __float2bfloat16_rn((float)rem);
                const uint32_t off = op_offset(r, c);
                memcpy(&img[(size_t)(2 * h) * kOpBytes + off], &hi, 2);
                memcpy(&img[(size_t)(2 * h + 1) * kOpBytes + off], &lo, 2);
            }
}

static size_t tc_smem_bytes() {
    return (size_t)kTileSmemOps + 1024 + 256 + std::max(sizeof(TileAux), sizeof(StepAux)) + 64;
}

// Tbf layout: [T image mb^2 x 64 KB | FP32 coefficients natom x P x 8 | error word | pad]
static size_t tbf_coef_off(const TiState &st) { return (size_t)st.tc_mb * st.tc_mb * 2 * kOpBytes; }
static size_t tbf_err_off(const TiState &st, int natom) {
    return tbf_coef_off(st) + (size_t)natom * st.P * 8 * sizeof(float);
}
static size_t tbf_fold_off(const TiState &st, int natom) { return tbf_err_off(st, natom) + 64; }
static size_t tbf_kbase_off(const TiState &st, int natom) {
    return tbf_fold_off(st, natom) + (size_t)natom * st.P * 8 * sizeof(float);
}
static size_t tbf_kscale_off(const TiState &st, int natom) {
    return tbf_kbase_off(st, natom) + (size_t)st.P * 8 * sizeof(float);
}

}  // namespace

int tc_built() { return 1; }

// 0: unsupported; 1: fused 64-column tiles (P = 128, one-atom 1-D or 2-D
// surface, Langevin); 2: blocked GEMMs (P <= 512 with P % 4 == 0, any surface,
// Langevin or Andersen).  dHdrlimit re-initialisation (a Langevin option) runs
// in the blocked form (force kernel flags, k_ti_reinit re-initialises).
int tc_supported(const TiState &st, const pg_ctx &ctx) {
    if (st.cfg.dhdr_limit >= 0.0 && st.cfg.thermostat == PG_LANGEVIN)
        return (st.P % 4 == 0 && st.P <= kMaxMb * kP && ctx.nd <= kMaxDof) ? 2 : 0;
    if (st.cfg.thermostat == PG_ANDERSEN) return (st.P % 4 == 0 && st.P <= kMaxMb * kP && ctx.nd <= kMaxDof) ? 2 : 0;
    if (st.P == kP && ctx.natom == 1 &&
        ((ctx.pes_id == PG_PES_2DTEST && ctx.nd == 2) || (ctx.pes_id == PG_PES_1D && ctx.nd == 1)))
        return 1;
    if (st.P % 4 == 0 && st.P <= kMaxMb * kP && ctx.nd <= kMaxDof) return 2;
    return 0;
}

// The persistent folded step (k_tf_step) applies to blocked batches with
// P = 256, the Langevin thermostat without dHdrlimit, and the 9-atom surface
// whose table lists its 36 pairs in order (evaluated unrolled, in registers).
int tf_supported(const TiState &st, const pg_ctx &ctx) {
    return st.P == kFP && st.cfg.thermostat == PG_LANGEVIN && st.cfg.dhdr_limit < 0.0 && ctx.canon9 &&
           ctx.fparams.size() <= (size_t)kTfParams;
}

// (p, q) <- R O R (p - dt g, q) as one map: R the half rotation [rA rB; rC rD],
// O the OU step p <- ou_a p + ou_s z, composed in FP64:
// [K11 K12 N1 K11 dt | K21 K22 N2 K21 dt].
static void fold_map(const ModeCoef &c, double dt, double (&o)[8]) {
    const double k11 = c.ou_a * c.rA * c.rA + c.rB * c.rC, k12 = c.ou_a * c.rA * c.rB + c.rB * c.rD;
    const double k21 = c.rC * (c.ou_a * c.rA + c.rD), k22 = c.ou_a * c.rB * c.rC + c.rD * c.rD;
    o[0] = k11;
    o[1] = k12;
    o[2] = c.rA * c.ou_s;
    o[3] = k11 * dt;
    o[4] = k21;
    o[5] = k22;
    o[6] = c.rC * c.ou_s;
    o[7] = k21 * dt;
}

// The folded step's update maps as a unit-mass map per mode (base, P x 8) and
// mass factors per atom (scale, natom x 4: m, sqrt m, 1 / m, 1 / sqrt m): with
// bead masses m (lambda_k tau)^2 the map of (atom, mode) is the mode's base
// times [1, m, sqrt m, 1 | 1 / m, 1, 1 / sqrt m, 1 / m].  Checked against the
// per-atom maps (relative 1e-9 in FP64); PG_ERR_STATE if they do not factor.
static int tf_mass_tables(const pg_ctx *ctx, const TiState &st, float *base, float *scale) {
    const int P = st.P, natom = ctx->natom;
    auto factors = [](double m, double (&f)[8]) {
        const double r = std::sqrt(m);
        const double v[8] = {1.0, m, r, 1.0, 1.0 / m, 1.0, 1.0 / r, 1.0 / m};
        for (int i = 0; i < 8; i++) f[i] = v[i];
    };
    double f0[8];
    factors(ctx->mass[0], f0);
    for (int k = 0; k < P; k++) {
        double b[8];
        fold_map(st.hcoef[(size_t)natom * k], st.cfg.dt, b);
        for (int i = 0; i < 8; i++) b[i] /= f0[i];
        for (int at = 0; at < natom; at++) {
            double o[8], f[8];
            fold_map(st.hcoef[(size_t)at + (size_t)natom * k], st.cfg.dt, o);
            factors(ctx->mass[at], f);
            for (int i = 0; i < 8; i++)
                if (!(std::fabs(o[i] - b[i] * f[i]) <= 1e-9 * std::fabs(o[i]) + 1e-300))
                    return fail(PG_ERR_STATE, "folded step: the update maps do not factor into mode and mass parts");
        }
        for (int i = 0; i < 8; i++) base[(size_t)k * 8 + i] = (float)b[i];
    }
    for (int at = 0; at < natom; at++) {
        const double m = ctx->mass[at], r = std::sqrt(m);
        scale[4 * at] = (float)m;
        scale[4 * at + 1] = (float)r;
        scale[4 * at + 2] = (float)(1.0 / m);
        scale[4 * at + 3] = (float)(1.0 / r);
    }
    return PG_OK;
}

// Tensor-core tables of a batch: the split image of T (rebuilt only when P or
// the buffer changes), the FP32 coefficient and folded-map tables (uploaded
// when they differ from the last upload), the error word, and the column table.
int tc_prepare(pg_ctx *ctx, TiState &st) {
    st.tc_mb = blocks_for(st.P);
    const int P = st.P;
    size_t ncoef = (size_t)ctx->natom * P * 8;
    const size_t nkb = (size_t)P * 8, nks = (size_t)ctx->natom * 4;
    size_t bytes = tbf_kscale_off(st, ctx->natom) + nks * sizeof(float);
    cudaError_t e = st.Tbf.ensure(bytes);
    if (e != cudaSuccess) return cuda_fail(e, "tensor-core tables");
    if (st.hcoef.size() != (size_t)ctx->natom * P) return fail(PG_ERR_STATE, "mode coefficients missing");
    const std::vector<ModeCoef> &mc = st.hcoef;
    // [coefficients | folded map | unit-mass coefficients | atom mass factors]
    std::vector<float> tabs(2 * ncoef + nkb + nks, 0.f);
    float *cf = tabs.data(), *fold = tabs.data() + ncoef, *kb = fold + ncoef, *ks = kb + nkb;
    for (int at = 0; at < ctx->natom; at++)
        for (int k = 0; k < P; k++) {
            const ModeCoef &c = mc[(size_t)at + (size_t)ctx->natom * k];
            float *o = &cf[((size_t)at * P + k) * 8];
            o[0] = (float)c.rA;
            o[1] = (float)c.rB;
            o[2] = (float)c.rC;
            o[3] = (float)c.rD;
            o[4] = (float)c.ou_a;
            o[5] = (float)c.ou_s;
            o[6] = (float)c.pscale;  // sqrt(beadmass / betan): Andersen momentum scale
        }
    for (int at = 0; at < ctx->natom; at++)
        for (int k = 0; k < P; k++) {
            double m8[8];
            fold_map(mc[(size_t)at + (size_t)ctx->natom * k], st.cfg.dt, m8);
            float *o = &fold[((size_t)at * P + k) * 8];
            for (int i = 0; i < 8; i++) o[i] = (float)m8[i];
        }
    // the coefficients of a unit mass: with bead masses m (lambda_k tau)^2, rA, rD and
    // ou_a do not depend on the atom, rB scales as m, rC as 1 / m, ou_s and pscale
    // as sqrt m (checked against every atom's coefficients)
    for (int k = 0; k < P; k++) {
        const ModeCoef &c0 = mc[(size_t)ctx->natom * k];
        const double m0 = ctx->mass[0], r0 = std::sqrt(m0);
        const double b[7] = {c0.rA, c0.rB / m0, c0.rC * m0, c0.rD, c0.ou_a, c0.ou_s / r0, c0.pscale / r0};
        for (int at = 0; at < ctx->natom; at++) {
            const ModeCoef &c = mc[(size_t)at + (size_t)ctx->natom * k];
            const double m = ctx->mass[at], r = std::sqrt(m);
            const double o[7] = {c.rA, c.rB, c.rC, c.rD, c.ou_a, c.ou_s, c.pscale};
            const double f[7] = {1.0, m, 1.0 / m, 1.0, 1.0, r, r};
            for (int i = 0; i < 7; i++)
                if (!(std::fabs(o[i] - b[i] * f[i]) <= 1e-9 * std::fabs(o[i]) + 1e-300))
                    return fail(PG_ERR_STATE, "blocked kick: the mode coefficients do not factor into mode and mass parts");
        }
        for (int i = 0; i < 7; i++) kb[(size_t)k * 8 + i] = (float)b[i];
    }
    for (int at = 0; at < ctx->natom; at++) {
        const double m = ctx->mass[at], r = std::sqrt(m);
        ks[4 * at] = (float)m;
        ks[4 * at + 1] = (float)r;
        ks[4 * at + 2] = (float)(1.0 / m);
        ks[4 * at + 3] = (float)(1.0 / r);
    }
    unsigned char *d = st.Tbf.as<unsigned char>();
    const bool same_buf = st.tc_img_ptr == (const void *)d;
    if (!same_buf || st.tc_img_P != P) {
        std::vector<unsigned char> img;
        build_split_image(P, img);
        PG_CUDA(cudaMemcpyAsync(d, img.data(), img.size(), cudaMemcpyHostToDevice, ctx->stream));
        PG_CUDA(cudaStreamSynchronize(ctx->stream));  // img is a local pageable buffer
        st.tc_img_P = P;
        st.tc_img_ptr = d;
        st.tc_tabs.clear();
    }
    if (st.tc_tabs != tabs) {
        PG_CUDA(cudaMemcpyAsync(d + tbf_coef_off(st), cf, ncoef * sizeof(float), cudaMemcpyHostToDevice,
                                ctx->stream));
        PG_CUDA(cudaMemcpyAsync(d + tbf_fold_off(st, ctx->natom), fold, (ncoef + nkb + nks) * sizeof(float),
                                cudaMemcpyHostToDevice, ctx->stream));
        PG_CUDA(cudaStreamSynchronize(ctx->stream));  // tabs is a local pageable buffer
        st.tc_tabs.swap(tabs);
    }
    PG_CUDA(cudaMemsetAsync(d + tbf_err_off(st, ctx->natom), 0, 64, ctx->stream));
    {
        const int64_t ncols = st.nrings * st.nd;
        e = st.tccol.ensure((size_t)ncols * 32);
        if (e != cudaSuccess) return cuda_fail(e, "tensor-core column table");
        unsigned char *cb = st.tccol.as<unsigned char>();
        k_tc_cols<<<(unsigned)((ncols + 255) / 256), 256, 0, ctx->stream>>>(
            ncols, st.nd, ctx->ndim, P, st.ringlam.as<int32_t>(), st.ringseed.as<uint64_t>(),
            st.ringstream.as<uint32_t>(), st.avec.as<double>(), st.bvec.as<double>(), st.dbdl.as<double>(),
            ctx->d_mass.as<double>(), reinterpret_cast<float *>(cb), reinterpret_cast<float *>(cb + 4 * ncols),
            reinterpret_cast<uint32_t *>(cb + 8 * ncols), reinterpret_cast<int32_t *>(cb + 12 * ncols),
            reinterpret_cast<uint64_t *>(cb + 16 * ncols), reinterpret_cast<double *>(cb + 24 * ncols));
        PG_CUDA(cudaGetLastError());
    }
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (!st.tc_attr) {
        size_t sm = tc_smem_bytes();
        PG_CUDA(cudaFuncSetAttribute(k_tc_step<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tc_step<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tc_step<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tc_step<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tc_final, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tb_pos, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tb_kick, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_tb_kick_nm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        st.tc_attr = true;
    }
    // the force kernel's shared memory depends on the surface and the dof count
    PG_CUDA(cudaFuncSetAttribute(k_tb_force, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tb_force_smem(st.nd, (int)ctx->fparams.size())));
    if (st.tf_fused) {
        // [folded image 128 KB | unit-mass maps P x 8 | atom mass factors natom x 4]
        const size_t nb = (size_t)kFP * 8, ns = (size_t)ctx->natom * 4;
        e = st.tfimg.ensure(kTfImg + (nb + ns) * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(e, "folded transform image");
        if (st.tf_img_ptr != st.tfimg.ptr) {  // written once per buffer
            std::vector<unsigned char> img;
            build_fold_image(img);
            PG_CUDA(cudaMemcpyAsync(st.tfimg.ptr, img.data(), img.size(), cudaMemcpyHostToDevice, ctx->stream));
            PG_CUDA(cudaStreamSynchronize(ctx->stream));  // img is a local pageable buffer
            st.tf_img_ptr = st.tfimg.ptr;
        }
        std::vector<float> mt(nb + ns);
        if (int rc = tf_mass_tables(ctx, st, mt.data(), mt.data() + nb)) return rc;
        PG_CUDA(cudaMemcpyAsync(st.tfimg.as<unsigned char>() + kTfImg, mt.data(), mt.size() * sizeof(float),
                                cudaMemcpyHostToDevice, ctx->stream));
        PG_CUDA(cudaStreamSynchronize(ctx->stream));  // mt is a local pageable buffer
        const int sm = (int)tf_step_smem_bytes(), so = (int)tf_out_smem_bytes();
        PG_CUDA(cudaFuncSetAttribute(k_tf_step<27, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
        PG_CUDA(cudaFuncSetAttribute(k_tf_out<27, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, so));
    }
    return PG_OK;
}

int32_t tc_error(pg_ctx *ctx, TiState &st) {
    const unsigned char *d = st.Tbf.as<unsigned char>();
    int32_t e = 0;
    if (cudaMemcpyAsync(&e, d + tbf_err_off(st, ctx->natom), sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream) !=
        cudaSuccess)
        return -1;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return -1;
    return e;
}

static void tc_make_args(pg_ctx *ctx, TiState &st, TcArgs &a, int &pesk) {
    memset(&a, 0, sizeof(a));
    a.nrings = st.nrings;
    a.nd = st.nd;
    a.ndim = ctx->ndim;
    a.natom = ctx->natom;
    a.dt = (float)st.cfg.dt;
    a.imin = st.cfg.imin;
    unsigned char *d = st.Tbf.as<unsigned char>();
    a.gT = d;
    a.coef = reinterpret_cast<const float *>(d + tbf_coef_off(st));
    a.err = reinterpret_cast<int32_t *>(d + tbf_err_off(st, ctx->natom));
    a.step0 = reinterpret_cast<const int64_t *>(st.red.as<double>() + 3 * st.nlambda);
    a.mass = ctx->d_mass.as<double>();
    a.avec = st.avec.as<double>();
    a.bvec = st.bvec.as<double>();
    a.dbdl = st.dbdl.as<double>();
    a.ringlam = st.ringlam.as<int32_t>();
    a.ringseed = st.ringseed.as<uint64_t>();
    a.ringstream = st.ringstream.as<uint32_t>();
    a.q = st.q.as<float>();
    a.pi = st.pi.as<float>();
    a.x = st.x.as<float>();
    a.acc = st.acc.as<RingAcc>();
    {
        const int64_t ncols = st.nrings * st.nd;
        unsigned char *cb = st.tccol.as<unsigned char>();
        a.cxa = reinterpret_cast<const float *>(cb);
        a.cxs = reinterpret_cast<const float *>(cb + 4 * ncols);
        a.cstream = reinterpret_cast<const uint32_t *>(cb + 8 * ncols);
        a.cjdof = reinterpret_cast<const int32_t *>(cb + 12 * ncols);
        a.cseed = reinterpret_cast<const uint64_t *>(cb + 16 * ncols);
        a.cwest = reinterpret_cast<const double *>(cb + 24 * ncols);
        a.fold = reinterpret_cast<const float *>(d + tbf_fold_off(st, ctx->natom));
    }
    pesk = ctx->pes_id == PG_PES_2DTEST ? 2 : 1;
    const std::vector<double> &p = ctx->params;
    if (pesk == 2) {
        int m = p.size() >= 4 ? (int)p[0] : 6;
        double a0 = p.size() >= 4 ? p[1] : 2.0, b0 = p.size() >= 4 ? p[2] : 0.2, rho0 = p.size() >= 4 ? p[3] : 3.0;
        a.nwell = m;
        for (int k = 0; k < m; k++) {
            a.wc[2 * k] = (float)(rho0 * std::cos((double)(k + 1) * 2.0 * kPiRef / (double)m));
            a.wc[2 * k + 1] = (float)(rho0 * std::sin((double)(k + 1) * 2.0 * kPiRef / (double)m));
        }
        a.a0 = (float)a0;
        a.b0 = (float)b0;
        a.pow10 = ((float)a0 == 10.0f * (float)b0) ? 1 : 0;
    } else {
        a.H = p.size() >= 2 ? (float)p[0] : 1.0f;
        a.x0 = p.size() >= 2 ? (float)p[1] : 1.0f;
    }
}

static unsigned tc_grid(const TiState &st) { return (unsigned)((st.nrings * st.nd + kNc - 1) / kNc); }

// Step i of an advance (k_tc_step), or the final pass after n steps (k_tc_final).
static int tc_launch_step(pg_ctx *ctx, TiState &st, int64_t i, int nsub, cudaStream_t s) {
    TcArgs a;
    int pesk;
    tc_make_args(ctx, st, a, pesk);
    a.sofs = i;
    a.do_est = i > 0 ? 1 : 0;
    a.nsub = nsub;
    const size_t sm = tc_smem_bytes();
    // persistent: two CTAs per SM (the shared-memory limit), equal ring ranges
    const unsigned grid = (unsigned)std::min<int64_t>(2 * (int64_t)(ctx->sm_count > 0 ? ctx->sm_count : 1),
                                                      (int64_t)tc_grid(st));
    // programmatic serialization: this launch's set-up overlaps the tail of the
    // previous one (the kernel waits for it before touching the ring state)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kTileThreads);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // q resident in tensor memory when no CTA holds more than two chunks
    const int64_t rpc = kNc / st.nd, maxr = (st.nrings + grid - 1) / grid;
    const bool qt = (maxr + rpc - 1) / rpc <= 2;
    cudaError_t e;
    if (pesk == 2)
        e = qt ? cudaLaunchKernelEx(&cfg, k_tc_step<2, true>, a) : cudaLaunchKernelEx(&cfg, k_tc_step<2, false>, a);
    else
        e = qt ? cudaLaunchKernelEx(&cfg, k_tc_step<1, true>, a) : cudaLaunchKernelEx(&cfg, k_tc_step<1, false>, a);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "k_tc_step launch");
}

static int tc_launch_final(pg_ctx *ctx, TiState &st, int64_t n, cudaStream_t s) {
    TcArgs a;
    int pesk;
    tc_make_args(ctx, st, a, pesk);
    a.sofs = n;
    a.do_est = n > 0 ? 1 : 0;
    k_tc_final<<<tc_grid(st), kTileThreads, tc_smem_bytes(), s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_tc_final launch");
    k_tc_step_add<<<1, 1, 0, s>>>(const_cast<int64_t *>(a.step0), n);
    e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "step counter launch");
}

static void tb_make_args(pg_ctx *ctx, TiState &st, TbArgs &a) {
    memset(&a, 0, sizeof(a));
    a.nrings = st.nrings;
    a.nd = st.nd;
    a.ndim = ctx->ndim;
    a.natom = ctx->natom;
    a.P = st.P;
    a.mb = st.tc_mb;
    a.dt = (float)st.cfg.dt;
    a.imin = st.cfg.imin;
    unsigned char *d = st.Tbf.as<unsigned char>();
    a.gT = d;
    a.coef = reinterpret_cast<const float *>(d + tbf_coef_off(st));
    a.kbase = reinterpret_cast<const float *>(d + tbf_kbase_off(st, ctx->natom));
    a.kscale = reinterpret_cast<const float4 *>(d + tbf_kscale_off(st, ctx->natom));
    a.err = reinterpret_cast<int32_t *>(d + tbf_err_off(st, ctx->natom));
    a.step0 = reinterpret_cast<const int64_t *>(st.red.as<double>() + 3 * st.nlambda);
    a.mass = ctx->d_mass.as<double>();
    a.avec = st.avec.as<double>();
    a.bvec = st.bvec.as<double>();
    a.dbdl = st.dbdl.as<double>();
    a.ringlam = st.ringlam.as<int32_t>();
    a.ringseed = st.ringseed.as<uint64_t>();
    a.ringstream = st.ringstream.as<uint32_t>();
    a.q = st.q.as<float>();
    a.pi = st.pi.as<float>();
    a.x = st.x.as<float>();
    a.f = st.f.as<float>();
    a.acc = st.acc.as<RingAcc>();
    a.pes = ctx->pes_args();
    a.Tf = reinterpret_cast<const float *>(st.T.as<double>() + (size_t)st.P * st.P);
    a.betan = st.betan;
    a.noutput = (double)st.cfg.noutput;
    a.kick = st.kickflag.as<uint8_t>();
    a.dhdr_limit = st.cfg.dhdr_limit;
}

// Blocked form: kernel k (0 positions, 1 forces / estimator, 2 kick) of step
// offset i; final = the positions and estimator pass after the last step.
static int tb_launch_kernel(pg_ctx *ctx, TiState &st, int k, int64_t i, bool final_pass, cudaStream_t s) {
    TbArgs a;
    tb_make_args(ctx, st, a);
    a.sofs = i;
    a.do_est = i > 0 ? 1 : 0;
    a.do_force = final_pass ? 0 : 1;
    const unsigned grid = (unsigned)((st.nrings * st.nd + kNc - 1) / kNc);
    if (k == 0)
        k_tb_pos<<<grid, kTileThreads, tc_smem_bytes(), s>>>(a);
    else if (k == 1)
        k_tb_force<<<(unsigned)((st.nrings * st.P + kForceThreads - 1) / kForceThreads), kForceThreads,
                     tb_force_smem(st.nd, a.pes.nparams + pes_fparams_extra(a.pes.id)), s>>>(a);
    else
        k_tb_kick<<<grid, kTileThreads, tc_smem_bytes(), s>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "blocked tensor-form launch");
}

// Andersen step i of the blocked form: schedule, resample + half rotation,
// positions, forces, T F kick + half rotation, estimator.
static int tb_launch_andersen_step(pg_ctx *ctx, TiState &st, int64_t i, cudaStream_t s) {
    TbArgs a;
    tb_make_args(ctx, st, a);
    a.sofs = i;
    a.do_est = 0;
    a.do_force = 1;
    const int64_t nel = st.nrings * st.nd * st.P;
    const unsigned grid = (unsigned)((st.nrings * st.nd + kNc - 1) / kNc);
    k_tb_and_sched<<<(unsigned)((st.nrings + 127) / 128), 128, 0, s>>>(a);
    k_tb_and_pre<<<(unsigned)((nel + 255) / 256), 256, 0, s>>>(a);
    k_tb_pos<<<grid, kTileThreads, tc_smem_bytes(), s>>>(a);
    k_tb_force<<<(unsigned)((st.nrings * st.P + kForceThreads - 1) / kForceThreads), kForceThreads,
                 tb_force_smem(st.nd, a.pes.nparams + pes_fparams_extra(a.pes.id)), s>>>(a);
    k_tb_kick_nm<<<grid, kTileThreads, tc_smem_bytes(), s>>>(a);
    k_tb_and_est<<<(unsigned)((st.nrings + 3) / 4), 128, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "blocked Andersen step launch");
}

static int tb_launch(pg_ctx *ctx, TiState &st, int64_t nsteps, cudaStream_t s) {
    if (st.cfg.thermostat == PG_ANDERSEN) {
        for (int64_t i = 0; i < nsteps; i++) {
            int rc = tb_launch_andersen_step(ctx, st, i, s);
            if (rc) return rc;
        }
        // positions after the last step for read-out (the estimator ran per step)
        TbArgs a;
        tb_make_args(ctx, st, a);
        a.sofs = nsteps;
        k_tb_pos<<<(unsigned)((st.nrings * st.nd + kNc - 1) / kNc), kTileThreads, tc_smem_bytes(), s>>>(a);
        k_tc_step_add<<<1, 1, 0, s>>>(const_cast<int64_t *>(a.step0), nsteps);
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? PG_OK : cuda_fail(e, "blocked Andersen final launch");
    }
    // dHdrlimit: after each estimator (step i - 1, in the force kernel of step
    // i, and of the last step in the final pass) the flagged rings are
    // re-initialised with their forces before the next kick
    const bool reinit = st.cfg.dhdr_limit >= 0.0;
    for (int64_t i = 0; i < nsteps; i++)
        for (int k = 0; k < 3; k++) {
            int rc = tb_launch_kernel(ctx, st, k, i, false, s);
            if (rc) return rc;
            if (k == 1 && reinit && i > 0 && (rc = ti_launch_reinit(ctx, st, i, s))) return rc;
        }
    for (int k = 0; k < 2; k++) {
        int rc = tb_launch_kernel(ctx, st, k, nsteps, true, s);
        if (rc) return rc;
    }
    if (reinit)
        if (int rc = ti_launch_reinit(ctx, st, nsteps, s)) return rc;
    TbArgs a;
    tb_make_args(ctx, st, a);
    k_tc_step_add<<<1, 1, 0, s>>>(const_cast<int64_t *>(a.step0), nsteps);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "step counter launch");
}

// Persistent folded step (P = 256): launches of up to tc_steps_per_launch()
// MD steps, one CTA per SM, then the read-out pass and the step counter.
static void tf_make_args(pg_ctx *ctx, TiState &st, TfArgs &f) {
    TcArgs a;
    int pesk;
    tc_make_args(ctx, st, a, pesk);
    memset(&f, 0, sizeof(f));
    f.nrings = st.nrings;
    f.nd = st.nd;
    f.ndim = ctx->ndim;
    f.imin = st.cfg.imin;
    f.gT = st.tfimg.as<unsigned char>();
    f.fold = a.fold;
    f.mbase = reinterpret_cast<const float *>(st.tfimg.as<unsigned char>() + kTfImg);
    f.ascale = reinterpret_cast<const float4 *>(st.tfimg.as<unsigned char>() + kTfImg + (size_t)kFP * 8 * sizeof(float));
    f.q = a.q;
    f.pi = a.pi;
    f.x = a.x;
    f.acc = a.acc;
    f.cxa = a.cxa;
    f.cxs = a.cxs;
    f.cseed = a.cseed;
    f.cstream = a.cstream;
    f.cjdof = a.cjdof;
    f.cwest = a.cwest;
    f.step0 = a.step0;
    f.err = a.err;
    f.pes = ctx->pes_args();
}

static int tf_launch_one(pg_ctx *ctx, TiState &st, int64_t sofs, int nsub, bool final_pass, cudaStream_t s) {
    TfArgs f;
    tf_make_args(ctx, st, f);
    f.sofs = sofs;
    f.nsub = nsub;
    f.do_est = (final_pass && sofs > 0) ? 1 : 0;
    const unsigned grid = (unsigned)std::min<int64_t>(ctx->sm_count > 0 ? ctx->sm_count : 1, st.nrings);
    const size_t sm = tf_step_smem_bytes(), so = tf_out_smem_bytes();
    if (final_pass)
        k_tf_out<27, 2><<<grid, kTfThreads, so, s>>>(f);
    else
        k_tf_step<27, 2><<<grid, kTpThreads, sm, s>>>(f);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, final_pass ? "k_tf_out launch" : "k_tf_step launch");
}

static int tf_launch(pg_ctx *ctx, TiState &st, int64_t nsteps, cudaStream_t s);

// MD steps per k_tc_step launch (the per-launch set-up, mainly the 64 KB copy
// of T into every CTA, is paid once per launch).
constexpr int kStepsPerLaunch = 50;
int tc_steps_per_launch(const TiState &st) { return st.tc_steps > 0 ? st.tc_steps : kStepsPerLaunch; }

// The read-out pass (positions, estimator of the last step) and the step counter.
static int tf_launch_final(pg_ctx *ctx, TiState &st, int64_t nsteps, cudaStream_t s) {
    int rc = tf_launch_one(ctx, st, nsteps, 1, true, s);
    if (rc) return rc;
    TcArgs a;
    int pesk;
    tc_make_args(ctx, st, a, pesk);
    k_tc_step_add<<<1, 1, 0, s>>>(const_cast<int64_t *>(a.step0), nsteps);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "step counter launch");
}

static int tf_launch(pg_ctx *ctx, TiState &st, int64_t nsteps, cudaStream_t s) {
    const int per = tc_steps_per_launch(st);
    for (int64_t i = 0; i < nsteps; i += per) {
        int rc = tf_launch_one(ctx, st, i, (int)std::min<int64_t>(per, nsteps - i), false, s);
        if (rc) return rc;
    }
    return tf_launch_final(ctx, st, nsteps, s);
}

int tc_launch(pg_ctx *ctx, TiState &st, int64_t, int64_t nsteps, cudaStream_t s) {
    if (nsteps < 0) return PG_OK;  // the HBM copy of the state is current after every advance
    if (st.tf_fused) return tf_launch(ctx, st, nsteps, s);
    if (st.tc_blocked) return tb_launch(ctx, st, nsteps, s);
    const int per = tc_steps_per_launch(st);
    for (int64_t i = 0; i < nsteps; i += per) {
        int rc = tc_launch_step(ctx, st, i, (int)std::min<int64_t>(per, nsteps - i), s);
        if (rc) return rc;
    }
    return tc_launch_final(ctx, st, nsteps, s);
}

// Per-kernel event timing of nsteps steps (direct launches, no graph):
// ms[0] = k_tc_step, ms[1] = k_tc_final.
// Blocked form: ms[0..2] = k_tb_pos, k_tb_force, k_tb_kick per launch over nsteps steps.
static int tb_kernel_times(pg_ctx *ctx, TiState &st, int64_t nsteps, double *ms, int64_t *count) {
    cudaStream_t s = ctx->stream;
    if (st.cfg.thermostat == PG_ANDERSEN) {  // one kind: the six-launch step
        cudaEvent_t e0, e1;
        PG_CUDA(cudaEventCreate(&e0));
        PG_CUDA(cudaEventCreate(&e1));
        PG_CUDA(cudaEventRecord(e0, s));
        int rc = tb_launch(ctx, st, nsteps, s);
        if (rc) return rc;
        PG_CUDA(cudaEventRecord(e1, s));
        PG_CUDA(cudaEventSynchronize(e1));
        float v = 0.f;
        PG_CUDA(cudaEventElapsedTime(&v, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ms[0] = v / (double)nsteps;
        count[0] = nsteps;
        ms[1] = ms[2] = 0.0;
        count[1] = count[2] = 0;
        return PG_OK;
    }
    std::vector<cudaEvent_t> ev(3 * nsteps + 1);
    for (auto &e : ev) PG_CUDA(cudaEventCreate(&e));
    PG_CUDA(cudaEventRecord(ev[0], s));
    for (int64_t i = 0; i < nsteps; i++)
        for (int k = 0; k < 3; k++) {
            int rc = tb_launch_kernel(ctx, st, k, i, false, s);
            if (rc) return rc;
            PG_CUDA(cudaEventRecord(ev[3 * i + k + 1], s));
        }
    for (int k = 0; k < 2; k++) {
        int rc = tb_launch_kernel(ctx, st, k, nsteps, true, s);
        if (rc) return rc;
    }
    TbArgs a;
    tb_make_args(ctx, st, a);
    k_tc_step_add<<<1, 1, 0, s>>>(const_cast<int64_t *>(a.step0), nsteps);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaStreamSynchronize(s));
    double t[3] = {0.0, 0.0, 0.0};
    for (int64_t i = 0; i < nsteps; i++)
        for (int k = 0; k < 3; k++) {
            float v = 0.f;
            PG_CUDA(cudaEventElapsedTime(&v, ev[3 * i + k], ev[3 * i + k + 1]));
            t[k] += v;
        }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 3; k++) {
        ms[k] = t[k] / (double)nsteps;
        count[k] = nsteps;
    }
    return PG_OK;
}

// Per-kernel event timing of nsteps steps (direct launches, no graph): ms[0] =
// k_tc_step per launch (count[0] launches of nsub[0] steps each; a shorter
// last launch is not timed), ms[1] = k_tc_final.
int tc_kernel_times(pg_ctx *ctx, TiState &st, int64_t nsteps, double *ms, int64_t *count, int *nsub) {
    if (st.tc_blocked && !st.tf_fused) {
        *nsub = 1;
        return tb_kernel_times(ctx, st, nsteps, ms, count);
    }
    const bool tf = st.tf_fused != 0;  // k_tf_step: the same launch structure as k_tc_step
    cudaStream_t s = ctx->stream;
    const int per = (int)std::min<int64_t>(tc_steps_per_launch(st), nsteps);
    const int64_t nl = (nsteps + per - 1) / per;
    std::vector<cudaEvent_t> ev(nl + 2);
    for (auto &e : ev) PG_CUDA(cudaEventCreate(&e));
    for (int64_t l = 0; l < nl; l++) {
        PG_CUDA(cudaEventRecord(ev[l], s));
        const int n = (int)std::min<int64_t>(per, nsteps - l * per);
        int rc = tf ? tf_launch_one(ctx, st, l * per, n, false, s) : tc_launch_step(ctx, st, l * per, n, s);
        if (rc) return rc;
    }
    PG_CUDA(cudaEventRecord(ev[nl], s));
    int rc = tf ? tf_launch_final(ctx, st, nsteps, s) : tc_launch_final(ctx, st, nsteps, s);  // with the counter add
    if (rc) return rc;
    PG_CUDA(cudaEventRecord(ev[nl + 1], s));
    PG_CUDA(cudaStreamSynchronize(s));
    const int64_t nfull = nsteps / per;  // launches of exactly `per` steps
    double t1 = 0.0;
    for (int64_t l = 0; l < nfull; l++) {
        float a = 0.f;
        PG_CUDA(cudaEventElapsedTime(&a, ev[l], ev[l + 1]));
        t1 += a;
    }
    float a2 = 0.f;
    PG_CUDA(cudaEventElapsedTime(&a2, ev[nl], ev[nl + 1]));
    for (auto &e : ev) cudaEventDestroy(e);
    ms[0] = nfull > 0 ? t1 / (double)nfull : 0.0;
    ms[1] = a2;
    count[0] = nfull;
    count[1] = 1;
    *nsub = per;
    return PG_OK;
}

int tc_nm_transform(pg_ctx *ctx, int64_t P, int64_t ncol, const double *in, double *out) {
    if (P != kP) return fail(PG_ERR_UNSUPPORTED, "tensor-core transform needs P = 128");
    std::vector<unsigned char> img;
    build_split_image((int)P, img);
    size_t n = (size_t)P * ncol;
    PG_CUDA(ctx->scratch_a.ensure(n * sizeof(double)));
    PG_CUDA(ctx->scratch_b.ensure(n * sizeof(double)));
    PG_CUDA(ctx->scratch_c.ensure(img.size() + 64));
    cudaStream_t s = ctx->stream;
    unsigned char *dimg = ctx->scratch_c.as<unsigned char>();
    int32_t *derr = reinterpret_cast<int32_t *>(dimg + img.size());
    PG_CUDA(cudaMemcpyAsync(dimg, img.data(), img.size(), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemsetAsync(derr, 0, sizeof(int32_t), s));
    PG_CUDA(cudaMemcpyAsync(ctx->scratch_a.ptr, in, n * sizeof(double), cudaMemcpyHostToDevice, s));
    size_t sm = (size_t)kSmemOps + 1024 + sizeof(TcShared) + 64;
    PG_CUDA(cudaFuncSetAttribute(k_tc_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    unsigned grid = (unsigned)((ncol + kRows - 1) / kRows);
    k_tc_transform<<<grid, 128, sm, s>>>(dimg, ctx->scratch_a.as<double>(), ctx->scratch_b.as<double>(), ncol, derr,
                                         (uint64_t)ctx->wait_ns);
    PG_CUDA(cudaGetLastError());
    int32_t herr = 0;
    PG_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaMemcpyAsync(out, ctx->scratch_b.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (herr) return fail(PG_ERR_NUMERIC, "tensor-core transform: a device wait exceeded the wait limit");
    return PG_OK;
}

}  // namespace pg

// ---------------------------------------------------------------- allocation-free transform
// Some callers cannot call cudaMalloc.  A Fortran or MPI host program often
// hands all of the GPU's memory to its own pool allocator at start-up and sizes
// every device array once, so a library allocation would fail or fragment that
// pool; other callers run inside a section where cudaMalloc's implicit device
// synchronisation is not allowed.  For them, pg_nm_transform_noalloc runs the
// split-BF16 tcgen05 transform on caller-owned device buffers and keeps its only
// scratch -- the 64 KB split-BF16 image of T and an error word -- in the static
// device array below, sized for P = 128 (every GPU that loads the library holds
// it until the process exits).  The first call on each device builds the image
// there (make that first call before any stream capture); calls that overlap on
// the GPU share the array and race.
namespace pg {
namespace {
constexpr size_t kNoAllocScratchBytes = 2 * (size_t)kOpBytes + 256;  // image + error word
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
constexpr int kMaxDevices = 64;
static void *g_noalloc_ptr[kMaxDevices];  // device address of g_noalloc_scratch, per device
static bool g_noalloc_ready[kMaxDevices];
static std::mutex g_noalloc_setup;  // one host thread at a time runs a device's set-up
}  // namespace
}  // namespace pg

extern "C" int pg_nm_transform_noalloc(int64_t P, int64_t ncol, const double *d_in, double *d_out,
                                       void *stream) {
    using namespace pg;
    if (P != kP)
        return fail(PG_ERR_ARG, "pg_nm_transform_noalloc: the static scratch holds one 128 x 128 split-BF16 "
                                "image, so P must be 128");
    if (ncol < 0 || ncol > (((int64_t)1 << 31) - 1) * kRows)  // grid.x <= 2^31 - 1
        return fail(PG_ERR_ARG, "pg_nm_transform_noalloc: bad ncol");
    if (ncol == 0) return PG_OK;
    if (!d_in || !d_out) return fail(PG_ERR_ARG, "pg_nm_transform_noalloc: NULL device buffer");
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(PG_ERR_ARG, "pg_nm_transform_noalloc: device index too large");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    {
        std::lock_guard<std::mutex> lock(g_noalloc_setup);
        if (!g_noalloc_ready[dev]) {
            // one-time set-up on this device (make it before any stream capture):
            // the host-side name of the array is not a device address; ask the runtime.
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            k_build_split_image<<<(kP * kP + 255) / 256, 256, 0, s>>>(reinterpret_cast<unsigned char *>(ptr));
            PG_CUDA(cudaGetLastError());
            PG_CUDA(cudaStreamSynchronize(s));
            size_t sm = (size_t)kSmemOps + 1024 + sizeof(TcShared) + 64;
            PG_CUDA(cudaFuncSetAttribute(k_tc_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            g_noalloc_ptr[dev] = ptr;
            g_noalloc_ready[dev] = true;
        }
    }
    unsigned char *img = reinterpret_cast<unsigned char *>(g_noalloc_ptr[dev]);
    int32_t *derr = reinterpret_cast<int32_t *>(img + 2 * kOpBytes);
    // the array keeps the previous call's contents: clear the error word
    PG_CUDA(cudaMemsetAsync(derr, 0, sizeof(int32_t), s));
    size_t sm = (size_t)kSmemOps + 1024 + sizeof(TcShared) + 64;
    unsigned grid = (unsigned)((ncol + kRows - 1) / kRows);
    k_tc_transform<<<grid, 128, sm, s>>>(img, d_in, d_out, ncol, derr, kWaitLimitNs);
    PG_CUDA(cudaGetLastError());
    int32_t herr = 0;
    PG_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (herr) return fail(PG_ERR_NUMERIC, "pg_nm_transform_noalloc: a barrier wait timed out");
    return PG_OK;
}
