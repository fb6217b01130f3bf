/*
 * mlp.cu -- the learned active-set proposal: a small MLP that, from an agent's
 * sorted neighbours and its preferred velocity, proposes which constraints
 * are active at the optimum of its ORCA linear program (ORCA.cpp:428-587).
 * The proposal is only a hint: the tick verifies it exactly and runs the full
 * incremental LP whenever the check fails (kernels.cu), so it never changes
 * the tick's results.
 *
 *   input  96 = 16 neighbours x (relative position / neighbour distance,
 *               relative velocity / 2, radius sum) + preferred velocity /
 *               LP radius, zero-padded from 82
 *   hidden 128 -> GELU -> 128 -> GELU
 *   output 160 classes (see ecmg_internal.h, kCls*)
 *
 * Inference: BF16 weights and activations on the 5th-generation tensor
 * cores (tcgen05.mma, FP32 accumulators in tensor memory), weights staged
 * once per CTA in shared memory in the MMA operand layout.  Training: FP32
 * master weights; every forward and backward GEMM on the tensor cores with
 * BF16 operands and FP32 accumulation (k_tc_gemm), the elementwise steps,
 * softmax cross-entropy and Adam in FP32.
 * This translation unit is not part of the parity-critical arithmetic.
 */
#include "../../include/ecmg.h"
#include "ecmg_internal.h"

#include <cuda.h> /* CUtensorMap (the encoder is reached through the runtime) */
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

using namespace ecmg;

namespace {

constexpr int IN = kMlpIn, HID = kMlpHid, OUT = kMlpOut;
__device__ __forceinline__ float gelu(float x)
{
    const float k0 = 0.7978845608028654f, k1 = 0.044715f; /* sqrt(2/pi), tanh approximation */
    return 0.5f * x * (1.0f + tanhf(k0 * (x + k1 * x * x * x)));
}

__device__ __forceinline__ float gelu_grad(float x)
{
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    float u = k0 * (x + k1 * x * x * x);
    float th = tanhf(u);
    float du = k0 * (1.0f + 3.0f * k1 * x * x);
    return 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * du;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi); /* .x = lo (low half), .y = hi */
    return *reinterpret_cast<uint32_t*>(&v);
}

/* ------------------------------------------------------------------------
 * Inference on the 5th-generation tensor cores (tcgen05).  One CTA of
 * sixteen warps per SM, persistent over tiles of 128 agents, as four
 * independent pipelines: warps 4g .. 4g+3 run the tiles of pipeline g, each
 * with its own operand tile in shared memory, its own 128 tensor-memory
 * columns and its own named barrier, so that the epilogues of some
 * pipelines run while another's MMA chain occupies the tensor core (the
 * epilogues, not the tensor core, bound the kernel).  Per tile four chains
 * (M = 128; N = 128 / 128 / 128 + 32, layer 3 in two chains over the same
 * columns; K = 96 / 128 / 128 in steps of 16), each issued by the
 * pipeline's first thread and completed through its mbarrier (FP32
 * accumulators, 128 lanes x N columns).  Epilogue: warp w reads lanes
 * 32 (w mod 4) .. +31 (its rows) with tcgen05.ld, the load of the next 16
 * columns in flight while the current ones are used -- bias + GELU
 * (tanh.approx) + BF16 into the operand tile, or bias + argmax over the 160
 * outputs (first maximum wins).  The operand tile holds the features (one
 * TMA copy), then each hidden layer over the operand the previous chain has
 * finished reading; the next tile's copy is requested when the last chain
 * of a tile has completed.  Operands sit in shared memory in the canonical
 * K-major layout without swizzle: 8-row x 16-byte core matrices; the row
 * groups of one 8-column chunk are adjacent (stride byte offset 128), chunks
 * R x 16 bytes apart (leading byte offset) for an operand of R rows.  One
 * chunk of a 128-row feature tile is one 2 KB TMA box (8 columns x 128
 * rows).  Every wait is bounded (spin limit); on a timeout the pipeline sets
 * the error bit, waits for its copy and MMA chain in flight, and the CTA
 * frees its tensor memory and returns.
 * ---------------------------------------------------------------------- */
constexpr int kTile = 128;      /* agents per tile (MMA M) */
constexpr int kGroups = 4;      /* independent pipelines per CTA */
constexpr int kSlotCols = 128;  /* tensor-memory columns per pipeline (layer 3 runs as N = 128 + 32) */
constexpr int kTmemCols = kGroups * kSlotCols;
constexpr int kInferThreads = 128 * kGroups;
constexpr int kOutA = 128;      /* layer-3 outputs of the first chain */
constexpr int kSpinDefault = 1 << 22;

/* byte offset of element (r, k) of an [R x K] bf16 operand in that layout */
__host__ __device__ constexpr int tc_off(int r, int k, int R)
{
    return ((k >> 3) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

constexpr int kW1B = HID * IN * 2, kW2B = HID * HID * 2, kW3B = OUT * HID * 2; /* B operands: N rows x K */
constexpr int kWB = kW1B + kW2B + kW3B;
constexpr int kXB = kTile * IN * 2, kHB = kTile * HID * 2;
/* weights, one operand tile per pipeline (the feature tile, then each hidden
   tile over it), biases, tensor-memory address and barriers */
constexpr size_t kInferSmem = (size_t)kWB + kGroups * kHB + sizeof(float) * (2 * HID + OUT) + 128;
static_assert(kXB <= kHB, "a feature tile fits the pipeline's operand tile");
static_assert(kInferSmem <= 232448, "shared memory of one CTA");

/* shared-memory matrix descriptor (no swizzle) */
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46; /* descriptor version */
    return d;                /* base offset 0, relative LBO, layout type 0: no swizzle */
}

/* instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D */
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* D[tmem] (+)= A[M x K] * B[K x N], K-steps of 16 (two chunks), one thread;
   B is N rows of an operand packed with R rows (R = N, or a row block of a
   taller operand: chunks R x 16 bytes apart) */
__device__ __forceinline__ void tc_layer(uint32_t tmem, uint32_t a_saddr, uint32_t b_saddr, int K, int N, int R)
{
    const uint32_t id = tc_idesc(kTile, N);
    for (int ks = 0; ks < K / 16; ks++) {
        const uint64_t ad = tc_sdesc(a_saddr + ks * 2 * (kTile * 16), kTile * 16, 128);
        const uint64_t bd = tc_sdesc(b_saddr + ks * 2 * (R * 16), R * 16, 128);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(id), "r"(acc));
    }
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

/* bounded wait for the mbarrier phase with the given parity: false after
   `limit` polls.  Limits of at least 1024 poll with try_wait (which may
   suspend the thread for a while); smaller ones -- the diagnostic setting
   of ecmg_mlp_set_wait_limit -- with the non-blocking test_wait, so that a
   limit of one poll really gives up at once */
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int limit = kSpinDefault)
{
    const bool blocking = limit >= 1024;
    for (int it = 0; it < limit; it++) {
        uint32_t ok;
        if (blocking)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(mbar), "r"(parity)
                : "memory");
        else
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(mbar), "r"(parity)
                : "memory");
        if (ok) return true;
    }
    return false;
}

/* 16 fp32 columns of this thread's lane, issued without waiting; the
   registers are valid after tmem_wait16 on them (the wait takes them as
   operands, so that no use is scheduled before it) */
__device__ __forceinline__ void tmem_issue16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait16(uint32_t (&r)[16])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}
/* f(registers, column) over `cols` columns (a multiple of 32) in chunks of
   16, the load of each chunk in flight while the previous one is used */
template <class F>
__device__ __forceinline__ void tmem_chunks(uint32_t taddr, int cols, F&& f)
{
    uint32_t ra[16], rb[16];
    tmem_issue16(taddr, ra);
    tmem_wait16(ra);
#pragma unroll 1
    for (int c = 0; c < cols; c += 32) {
        tmem_issue16(taddr + (uint32_t)(c + 16), rb);
        f(ra, c);
        tmem_wait16(rb);
        const bool more = c + 32 < cols;
        if (more) tmem_issue16(taddr + (uint32_t)(c + 32), ra);
        f(rb, c + 16);
        if (more) tmem_wait16(ra);
    }
}

/* W [K x N] row-major FP32 -> BF16 B operand (N rows x K) in the tc layout */
__global__ void k_pack_tc(const float* W, int K, int N, unsigned char* out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K * N; i += gridDim.x * blockDim.x) {
        int n = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(out + tc_off(n, k, N)) = __float2bfloat16_rn(W[(size_t)k * N + n]);
    }
}

/* the 12 TMA boxes (8 columns x 128 rows) of the feature tile at row r0 */
__device__ __forceinline__ void tma_tile(const CUtensorMap* tm, uint32_t sdst, int r0, uint32_t mbar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"((uint32_t)kXB)
                 : "memory");
#pragma unroll 1
    for (int kc = 0; kc < IN / 8; kc++)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
                "r"(sdst + (uint32_t)(kc * kTile * 16)),
            "l"(tm), "r"(kc * 8), "r"(r0), "r"(mbar)
            : "memory");
}

__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

/* GELU (tanh form) for inference: the hardware tanh approximation (relative
   error about 2^-11, below the BF16 rounding of the activations) */
__device__ __forceinline__ float gelu_fast(float x)
{
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    const float u = k0 * __fmaf_rn(k1 * (x * x), x, x);
    const float hx = 0.5f * x;
    return __fmaf_rn(hx, tanh_approx(u), hx);
}

/* 32 consecutive fp32 columns of this thread's lane, one wait */
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory"); /* the registers are tied to the wait: no use before it */
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

/* barrier of one 4-warp group (ids 1 and 2; 0 is the CTA barrier) */
__device__ __forceinline__ void group_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
/* barrier of one group that also ORs a flag over its threads */
__device__ __forceinline__ bool group_any(bool v, int id)
{
    unsigned r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, %2, 128, p;\nselp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((unsigned)v), "r"(id)
        : "memory");
    return r != 0;
}

/* class of every row of X [n, IN] (bf16, row-major); err |= errbit when a
   wait runs past `spin` polls (the CTA then drains and stops) */
__global__ void __launch_bounds__(kInferThreads, 1)
    k_mlp_infer(const __grid_constant__ CUtensorMap tmX, const int* n_ptr, int n_fixed, const unsigned char* wpack,
                const float* bias, unsigned char* cls, int* err, int errbit, int spin)
{
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* sW1 = sm;
    unsigned char* sW2 = sW1 + kW1B;
    unsigned char* sW3 = sW2 + kW2B;
    unsigned char* sT = sW3 + kW3B; /* [kGroups][kHB] operand tiles */
    float* sb = reinterpret_cast<float*>(sT + kGroups * kHB);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(sb + 2 * HID + OUT);
    uint64_t* s_mbar = reinterpret_cast<uint64_t*>(
        (reinterpret_cast<uintptr_t>(s_tmem + 2) + 7) & ~(uintptr_t)7); /* [g] MMA done, [kGroups + g] tile landed */
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = warp >> 2, quad = warp & 3, gt = tid & 127; /* pipeline, TMEM lane quarter, thread in group */
    const int bar_id = 1 + g;
    const int n = n_ptr ? *n_ptr : n_fixed;

    for (int i = tid; i < kWB / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(sm)[i] = reinterpret_cast<const uint4*>(wpack)[i];
    for (int i = tid; i < 2 * HID + OUT; i += blockDim.x) sb[i] = bias[i];
    const uint32_t mbar0 = (uint32_t)__cvta_generic_to_shared(s_mbar);
    if (tid == 0) {
        for (int b = 0; b < 2 * kGroups; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8u * b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    /* from here on the groups run independent pipelines */
    const uint32_t tmem = *s_tmem + (uint32_t)(g * kSlotCols);
    const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16);
    const uint32_t aT = (uint32_t)__cvta_generic_to_shared(sT + g * kHB);
    unsigned char* tbuf = sT + g * kHB;
    const uint32_t aW1 = (uint32_t)__cvta_generic_to_shared(sW1), aW2 = (uint32_t)__cvta_generic_to_shared(sW2),
                   aW3 = (uint32_t)__cvta_generic_to_shared(sW3);
    const uint32_t mb_mma = mbar0 + 8u * (uint32_t)g, mb_x = mbar0 + 8u * (uint32_t)(kGroups + g);
    const int row = quad * 32 + lane;
    const int ntiles = (n + kTile - 1) / kTile;
    int tile = (int)blockIdx.x + g * (int)gridDim.x; /* group g: tiles blockIdx.x + (kGroups j + g) gridDim.x */
    uint32_t ph_mma = 0u, ph_x = 0u;
    bool mma_pending = false, x_pending = false, fail = false;

    auto wait = [&](uint32_t mb, uint32_t& ph, bool& pending) {
        const bool ok = mbar_wait(mb, ph, spin);
        fail = group_any(!ok, bar_id);
        if (!fail) {
            ph ^= 1u;
            pending = false;
        }
        tc_fence_after();
        return !fail;
    };
    /* the operands the group's threads wrote are visible to the tensor core
       and the accumulator has been read out; then the leader issues one
       chain */
    auto mma = [&](uint32_t w, int K, int N, int R) {
        fence_async_smem();
        tc_fence_before();
        group_sync(bar_id);
        tc_fence_after();
        if (gt == 0) {
            tc_layer(tmem, aT, w, K, N, R);
            tc_commit(mb_mma);
        }
        mma_pending = true;
    };
    /* bias + GELU + BF16 of the accumulator into the group's operand tile
       (the chain that read it has completed) */
    auto epi_hidden = [&](const float* bl) {
        tmem_chunks(lane_base, HID, [&](uint32_t (&r)[16], int c) {
            const float4* b4 = reinterpret_cast<const float4*>(bl + c); /* 16-byte aligned */
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const float4 ba = b4[2 * q], bb = b4[2 * q + 1];
                const float* v = reinterpret_cast<const float*>(r) + 8 * q;
                uint4 u;
                u.x = pack_bf16(gelu_fast(v[0] + ba.x), gelu_fast(v[1] + ba.y));
                u.y = pack_bf16(gelu_fast(v[2] + ba.z), gelu_fast(v[3] + ba.w));
                u.z = pack_bf16(gelu_fast(v[4] + bb.x), gelu_fast(v[5] + bb.y));
                u.w = pack_bf16(gelu_fast(v[6] + bb.z), gelu_fast(v[7] + bb.w));
                *reinterpret_cast<uint4*>(tbuf + tc_off(row, c + 8 * q, kTile)) = u;
            }
        });
    };
    /* bias + running argmax over outputs [o0, o0 + cols); the first maximum wins */
    auto epi_argmax = [&](int o0, int cols, float& best, int& bi) {
        const float* bl = sb + 2 * HID + o0;
        tmem_chunks(lane_base, cols, [&](uint32_t (&r)[16], int c) {
            const float4* b4 = reinterpret_cast<const float4*>(bl + c); /* 16-byte aligned */
#pragma unroll
            for (int i = 0; i < 16; i += 4) {
                const float4 b = b4[i / 4];
                const float z0 = __uint_as_float(r[i]) + b.x, z1 = __uint_as_float(r[i + 1]) + b.y;
                const float z2 = __uint_as_float(r[i + 2]) + b.z, z3 = __uint_as_float(r[i + 3]) + b.w;
                if (z0 > best) { best = z0; bi = o0 + c + i; }
                if (z1 > best) { best = z1; bi = o0 + c + i + 1; }
                if (z2 > best) { best = z2; bi = o0 + c + i + 2; }
                if (z3 > best) { best = z3; bi = o0 + c + i + 3; }
            }
        });
    };

    if (tile < ntiles) {
        if (gt == 0) tma_tile(&tmX, aT, tile * kTile, mb_x);
        x_pending = true;
    }
    while (!fail && tile < ntiles) {
        if (!wait(mb_x, ph_x, x_pending)) break;
        mma(aW1, IN, HID, HID);
        if (!wait(mb_mma, ph_mma, mma_pending)) break;
        epi_hidden(sb);
        mma(aW2, HID, HID, HID);
        if (!wait(mb_mma, ph_mma, mma_pending)) break;
        epi_hidden(sb + HID);
        /* layer 3: outputs 0..127, read out, then 128..159 in the same columns */
        mma(aW3, HID, kOutA, OUT);
        if (!wait(mb_mma, ph_mma, mma_pending)) break;
        float best = -INFINITY;
        int bi = 0;
        epi_argmax(0, kOutA, best, bi);
        mma(aW3 + (uint32_t)(kOutA / 8) * 128u, HID, OUT - kOutA, OUT);
        if (!wait(mb_mma, ph_mma, mma_pending)) break;
        epi_argmax(kOutA, OUT - kOutA, best, bi);
        const int r = tile * kTile + row;
        if (r < n) cls[r] = (unsigned char)bi;
        /* the operand tile is free (the last chain has completed): the
           group's next features go into it */
        tile += kGroups * (int)gridDim.x;
        if (tile < ntiles) {
            if (gt == 0) tma_tile(&tmX, aT, tile * kTile, mb_x);
            x_pending = true;
        }
    }
    if (fail && gt == 0) atomicOr(err, errbit);
    /* nothing in flight may outlive the CTA: the group's copy and MMA chain
       are waited for (with the default bound) before tensor memory is freed */
    if (x_pending) (void)mbar_wait(mb_x, ph_x);
    if (mma_pending) (void)mbar_wait(mb_mma, ph_mma);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*s_tmem), "r"(kTmemCols) : "memory");
}

/* ------------------------------------------------------------------------
 * Training GEMMs on the tensor cores.  C[M x N] = A[M x K] * B[N x K]^T with
 * A and B BF16 row-major (K contiguous) in global memory, read by TMA in
 * stages of 64 K columns (8 boxes of 8 columns x 128 rows for A, 8 boxes of
 * 8 columns x N rows for B) into the canonical K-major layout, three stages
 * in flight; one thread issues the tcgen05.mma chain (M = 128, N <= 256,
 * K-steps of 16) into an FP32 accumulator in tensor memory; each warp reads
 * its 32 rows back for the epilogue: a plain FP32 store, or an atomic add
 * when the K range is split over CTAs (weight gradients, where K is the
 * batch).  Rows or columns beyond the tensors read as zeros.  Bounded waits
 * as in the inference kernel.
 * ---------------------------------------------------------------------- */
constexpr int kGemmStages = 3;
constexpr int kGemmKC = 64;                         /* K columns per stage */
constexpr int kGemmAB = kTile * kGemmKC * 2;        /* A bytes per stage (16 KB) */
constexpr int kGemmBB = 256 * kGemmKC * 2;          /* B bytes per stage, N <= 256 (32 KB) */
constexpr int kGemmStageB = kGemmAB + kGemmBB;
constexpr size_t kGemmSmem = (size_t)kGemmStages * kGemmStageB + 8 * (2 * kGemmStages + 1) + 16;

__device__ __forceinline__ void tma_box(const CUtensorMap* tm, uint32_t sdst, int x, int y, uint32_t mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(sdst), "l"(tm), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

__global__ void __launch_bounds__(128, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N, int K,
              int kper, float* C, int ldc, int atomic, int* err, int spin)
{
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTile;
    const int k0 = blockIdx.y * kper, k1 = min(K, k0 + kper);
    const int nch = k1 > k0 ? (k1 - k0 + kGemmKC - 1) / kGemmKC : 0;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t bar0 = sbase + (uint32_t)(kGemmStages * kGemmStageB);
    auto full = [&](int st) { return bar0 + 8u * (uint32_t)st; };
    auto empty = [&](int st) { return bar0 + 8u * (uint32_t)(kGemmStages + st); };
    const uint32_t done = bar0 + 8u * (uint32_t)(2 * kGemmStages);
    if (tid == 0) {
        for (int b = 0; b < 2 * kGemmStages + 1; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u * b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&s_tmem)),
                     "r"(256)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    if (tid == 0 && nch > 0) {
        uint32_t fph[kGemmStages] = {}, eph[kGemmStages] = {};
        bool xpend[kGemmStages] = {};
        const uint32_t bytes = (uint32_t)(kGemmAB + N * kGemmKC * 2);
        const uint32_t id = tc_idesc(kTile, N);
        auto load = [&](int c) {
            const int st = c % kGemmStages;
            const uint32_t a = sbase + (uint32_t)(st * kGemmStageB), b = a + (uint32_t)kGemmAB;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full(st)), "r"(bytes)
                         : "memory");
#pragma unroll 1
            for (int kc = 0; kc < kGemmKC / 8; kc++) {
                const int x = k0 + c * kGemmKC + kc * 8;
                tma_box(&tmA, a + (uint32_t)(kc * kTile * 16), x, m0, full(st));
                tma_box(&tmB, b + (uint32_t)(kc * N * 16), x, 0, full(st));
            }
            xpend[st] = true;
        };
        for (int c = 0; c < nch && c < kGemmStages; c++) load(c);
        bool fail = false;
        for (int c = 0; c < nch && !fail; c++) {
            const int st = c % kGemmStages;
            if (!mbar_wait(full(st), fph[st], spin)) { fail = true; break; }
            fph[st] ^= 1u;
            xpend[st] = false;
            tc_fence_after();
            const uint32_t a = sbase + (uint32_t)(st * kGemmStageB), b = a + (uint32_t)kGemmAB;
#pragma unroll
            for (int ks = 0; ks < kGemmKC / 16; ks++) {
                const uint64_t ad = tc_sdesc(a + (uint32_t)(ks * 2 * kTile * 16), kTile * 16, 128);
                const uint64_t bd = tc_sdesc(b + (uint32_t)(ks * 2 * N * 16), (uint32_t)N * 16, 128);
                const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(id), "r"(acc));
            }
            tc_commit(empty(st));
            /* refill the previous stage once its MMAs have read it */
            const int pc = c - 1;
            if (pc >= 0 && pc + kGemmStages < nch) {
                const int ps = pc % kGemmStages;
                if (!mbar_wait(empty(ps), eph[ps], spin)) { fail = true; break; }
                eph[ps] ^= 1u;
                load(pc + kGemmStages);
            }
        }
        /* every MMA issued so far completes on `done` (also after a timeout:
           nothing may be in flight when the CTA frees its tensor memory) */
        tc_commit(done);
        if (fail) {
            for (int st = 0; st < kGemmStages; st++)
                if (xpend[st]) (void)mbar_wait(full(st), fph[st]);
            (void)mbar_wait(done, 0u);
            s_fail = 1;
        }
    }
    __syncthreads();
    bool fail = s_fail != 0;
    if (!fail && nch > 0) {
        const bool ok = mbar_wait(done, 0u, spin);
        fail = __syncthreads_or(!ok) != 0;
        if (fail && tid == 0) (void)mbar_wait(done, 0u);
    }
    tc_fence_after();
    if (!fail && nch > 0) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t lb = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < N; c += 32) {
            float v[32];
            tmem_ld32(lb + (uint32_t)c, v);
            if (row < M) {
                float* out = C + (size_t)row * ldc + c;
                if (atomic) {
#pragma unroll
                    for (int i = 0; i < 32; i++) atomicAdd(out + i, v[i]);
                } else {
#pragma unroll
                    for (int i = 0; i < 32; i += 4) *reinterpret_cast<float4*>(out + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                }
            }
        }
    }
    if (fail && tid == 0) atomicOr(err, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256) : "memory");
}

/* the minibatch: rows of X (BF16) gathered by idx or by a seeded hash */
__global__ void k_gather(const __nv_bfloat16* X, const unsigned char* y, int n, int B, unsigned long long seed,
                         const int* idx, __nv_bfloat16* xb, int* yb)
{
    int r = blockIdx.x;
    if (r >= B) return;
    int src;
    if (idx) src = idx[r];
    else {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(r + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        src = (int)(z % (unsigned long long)n);
    }
    for (int c = threadIdx.x; c < IN; c += blockDim.x) xb[(size_t)r * IN + c] = X[(size_t)src * IN + c];
    if (threadIdx.x == 0) yb[r] = y[src];
}

/* elementwise steps between the GEMMs, in 32 x 32 tiles so that the
   transposed BF16 copy (the operand of a weight-gradient GEMM, [cols][ldT])
   is written coalesced as well:
     kPostGelu  Z += bias (kept for the backward pass), out = gelu(Z)
     kPostBack  D *= gelu'(Zs) (kept in place for the bias gradient), out = D
     kPostCopy  out = D (FP32 or BF16 input)
   out (BF16 row-major) and outT (BF16 transposed) may be null */
enum { kPostGelu = 0, kPostBack = 1, kPostCopy = 2 };
template <class TIn>
__global__ void k_post(TIn* D, const float* Zs, const float* bias, int rows, int cols, int mode, __nv_bfloat16* out,
                       __nv_bfloat16* outT, int ldT)
{
    __shared__ float tile[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = r0 + ty + 8 * i, c = c0 + tx;
        float v = 0.0f;
        if (r < rows && c < cols) {
            const size_t o = (size_t)r * cols + c;
            v = (float)D[o];
            if (mode == kPostGelu) {
                v += bias[c];
                D[o] = (TIn)v;
                v = gelu(v);
            } else if (mode == kPostBack) {
                v *= gelu_grad(Zs[o]);
                D[o] = (TIn)v;
            }
            if (out) out[o] = __float2bfloat16_rn(v);
        }
        tile[ty + 8 * i][tx] = v;
    }
    if (!outT) return;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int c = c0 + ty + 8 * i, r = r0 + tx;
        if (r < rows && c < cols) outT[(size_t)c * ldT + r] = __float2bfloat16_rn(tile[tx][ty + 8 * i]);
    }
}

/* BF16 copies of the master weights for the GEMM operands: W^T ([N][K],
   forward) and W as stored ([K][N] = the backward B operand) */
__global__ void k_wconv(const float* W, int K, int N, __nv_bfloat16* WT, __nv_bfloat16* Wn)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K * N; i += gridDim.x * blockDim.x) {
        const int k = i / N, n = i % N;
        const __nv_bfloat16 v = __float2bfloat16_rn(W[i]);
        if (WT) WT[(size_t)n * K + k] = v;
        if (Wn) Wn[i] = v;
    }
}

__global__ void k_bias_act(float* Z, float* Aout, const float* b, int rows, int cols, int act)
{
    size_t total = (size_t)rows * cols;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        float z = Z[i] + b[i % cols];
        Z[i] = z;
        if (Aout) Aout[i] = act ? gelu(z) : z;
    }
}

/* softmax cross-entropy: dZ = (softmax - onehot) / B, loss summed in *loss */
__global__ void k_softmax_ce(const float* Z, const int* y, int B, float* dZ, float* loss, int* correct)
{
    int r = blockIdx.x * blockDim.y + threadIdx.y;
    if (r >= B) return;
    const float* z = Z + (size_t)r * OUT;
    int lane = threadIdx.x;
    float mx = -INFINITY;
    int am = 0;
    for (int c = lane; c < OUT; c += 32)
        if (z[c] > mx) { mx = z[c]; am = c; }
    for (int o = 16; o; o >>= 1) {
        float om = __shfl_xor_sync(0xffffffffu, mx, o);
        int oa = __shfl_xor_sync(0xffffffffu, am, o);
        if (om > mx || (om == mx && oa < am)) { mx = om; am = oa; }
    }
    float se = 0.0f;
    for (int c = lane; c < OUT; c += 32) se += expf(z[c] - mx);
    for (int o = 16; o; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
    int yy = y[r];
    for (int c = lane; c < OUT; c += 32) {
        float p = expf(z[c] - mx) / se;
        dZ[(size_t)r * OUT + c] = (p - (c == yy ? 1.0f : 0.0f)) / (float)B;
    }
    if (lane == 0) {
        atomicAdd(loss, -(z[yy] - mx - logf(se)));
        if (correct && am == yy) atomicAdd(correct, 1);
    }
}

/* db[c] += sum over a chunk of rows of dZ[r][c] (db zeroed by the caller;
   grid.y chunks of rows) */
__global__ void k_colsum(const float* dZ, int rows, int cols, float* db)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    int chunk = (rows + gridDim.y - 1) / gridDim.y;
    int r0 = blockIdx.y * chunk, r1 = min(rows, r0 + chunk);
    float s = 0.0f;
    for (int r = r0; r < r1; r++) s += dZ[(size_t)r * cols + c];
    atomicAdd(&db[c], s);
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

/* parameter layout in one FP32 array: W1 [IN x HID], b1, W2 [HID x HID], b2, W3 [HID x OUT], b3 */
constexpr int OW1 = 0, OB1 = OW1 + IN * HID, OW2 = OB1 + HID, OB2 = OW2 + HID * HID, OW3 = OB2 + HID,
              OB3 = OW3 + HID * OUT, NPARAM = OB3 + OUT;

struct ecmg_mlp {
    float* p = nullptr;     /* FP32 master parameters */
    float* g = nullptr;     /* gradients */
    float* m = nullptr;     /* Adam first moment */
    float* v = nullptr;     /* Adam second moment */
    unsigned char* pack = nullptr; /* BF16 weights in the tensor-core operand layout (inference) */
    int* derr = nullptr;           /* inference error flag (ecmg_mlp_predict) */
    int spin = kSpinDefault;       /* polls of an mbarrier before the inference gives up */
    float* bias = nullptr;  /* b1 | b2 | b3 */
    int step = 0;
    bool packed = false;
    /* training scratch for batch B (transposed copies have rows of capT) */
    int cap = 0, capT = 0;
    float *z1 = nullptr, *z2 = nullptr, *z3 = nullptr, *dz3 = nullptr, *d2 = nullptr, *d1 = nullptr, *loss = nullptr;
    __nv_bfloat16 *xb = nullptr, *xT = nullptr, *a1 = nullptr, *a1T = nullptr, *a2 = nullptr, *a2T = nullptr,
                  *dz3h = nullptr, *dz3T = nullptr, *d2h = nullptr, *d2T = nullptr, *d1T = nullptr;
    /* BF16 operand copies of the weights: W^T for the forward GEMMs, W for the backward ones */
    __nv_bfloat16 *w1T = nullptr, *w2T = nullptr, *w3T = nullptr, *w2n = nullptr, *w3n = nullptr;
    int *yb = nullptr, *correct = nullptr, *gerr = nullptr;
    cudaStream_t s = nullptr;
};

namespace ecmg {
/* used by the tick (ctx.cu) */
cudaError_t mlp_infer(ecmg_mlp* mlp, const void* X, const int* n_dev, int n_max, unsigned char* cls, cudaStream_t s,
                      int sms, int* err, int errbit);
cudaError_t mlp_pack(ecmg_mlp* mlp);
}  // namespace ecmg

cudaError_t ecmg::mlp_pack(ecmg_mlp* mm)
{
    /* outside any stream capture: the inference kernel's shared memory limit */
    cudaError_t ea = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
    if (ea != cudaSuccess) return ea;
    if (mm->packed) return cudaSuccess;
    k_pack_tc<<<64, 256, 0, mm->s>>>(mm->p + OW1, IN, HID, mm->pack);
    k_pack_tc<<<64, 256, 0, mm->s>>>(mm->p + OW2, HID, HID, mm->pack + kW1B);
    k_pack_tc<<<64, 256, 0, mm->s>>>(mm->p + OW3, HID, OUT, mm->pack + kW1B + kW2B);
    cudaMemcpyAsync(mm->bias, mm->p + OB1, sizeof(float) * HID, cudaMemcpyDeviceToDevice, mm->s);
    cudaMemcpyAsync(mm->bias + HID, mm->p + OB2, sizeof(float) * HID, cudaMemcpyDeviceToDevice, mm->s);
    cudaMemcpyAsync(mm->bias + 2 * HID, mm->p + OB3, sizeof(float) * OUT, cudaMemcpyDeviceToDevice, mm->s);
    cudaError_t e = cudaStreamSynchronize(mm->s);
    if (e == cudaSuccess) mm->packed = true;
    return e;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

/* the driver's tensor-map encoder, reached through the runtime (no link
   against the driver library) */
static EncodeTiledFn tensor_map_encoder()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        cudaGetLastError();
    });
    return fn;
}

/* X [rows, IN] bf16 row-major as a 2D tensor; boxes of 8 columns x 128 rows,
   rows beyond `rows` read as zeros */
static cudaError_t feature_map(CUtensorMap* tm, const void* X, int rows)
{
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)IN, (cuuint64_t)(rows > 0 ? rows : 1)};
    const cuuint64_t strides[1] = {(cuuint64_t)IN * 2};
    const cuuint32_t box[2] = {8, (cuuint32_t)kTile};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(X), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t ecmg::mlp_infer(ecmg_mlp* mm, const void* X, const int* n_dev, int n_max, unsigned char* cls,
                            cudaStream_t s, int sms, int* err, int errbit)
{
    CUtensorMap tm;
    cudaError_t e = feature_map(&tm, X, n_max);
    if (e != cudaSuccess) return e;
    int tiles = (n_max + kTile - 1) / kTile;
    int grid = tiles < sms ? tiles : sms; /* one CTA per SM holds the weights once */
    if (grid < 1) grid = 1;
    k_mlp_infer<<<grid, kInferThreads, kInferSmem, s>>>(tm, n_dev, n_max, mm->pack, mm->bias, cls, err, errbit,
                                                         mm->spin);
    return cudaGetLastError();
}

extern "C" {

ecmg_status ecmg_mlp_create(unsigned long long seed, ecmg_mlp** out)
{
    if (!out) return ECMG_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return ECMG_ERR_NO_DEVICE;
    }
    ecmg_mlp* mm = new ecmg_mlp();
    bool ok = cudaStreamCreateWithFlags(&mm->s, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&mm->p, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&mm->g, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&mm->m, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&mm->v, sizeof(float) * NPARAM) == cudaSuccess &&
              cudaMalloc(&mm->pack, (size_t)kWB) == cudaSuccess &&
              cudaMalloc(&mm->derr, sizeof(int)) == cudaSuccess &&
              cudaMalloc(&mm->bias, sizeof(float) * (2 * HID + OUT)) == cudaSuccess &&
              cudaMalloc(&mm->loss, sizeof(float)) == cudaSuccess && cudaMalloc(&mm->correct, sizeof(int)) == cudaSuccess;
    if (!ok) {
        ecmg_mlp_destroy(mm);
        return ECMG_ERR_CUDA;
    }
    /* He-style init from a 64-bit mixer of the seed (host, deterministic) */
    std::vector<float> h(NPARAM, 0.0f);
    unsigned long long st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto rnd = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        unsigned long long z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0; /* U(-1,1) */
    };
    auto fill = [&](int off, int fan_in, int cnt) {
        double a = std::sqrt(3.0 * 2.0 / fan_in);
        for (int i = 0; i < cnt; i++) h[off + i] = (float)(a * rnd());
    };
    fill(OW1, IN, IN * HID);
    fill(OW2, HID, HID * HID);
    fill(OW3, HID, HID * OUT);
    cudaMemcpy(mm->p, h.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
    cudaMemset(mm->m, 0, sizeof(float) * NPARAM);
    cudaMemset(mm->v, 0, sizeof(float) * NPARAM);
    *out = mm;
    return ECMG_OK;
}

ecmg_status ecmg_mlp_destroy(ecmg_mlp* mm)
{
    if (!mm) return ECMG_ERR_INVALID_ARG;
    if (mm->s) cudaStreamSynchronize(mm->s);
    float* fs[] = {mm->p, mm->g, mm->m, mm->v, mm->bias, mm->z1, mm->z2, mm->z3, mm->dz3, mm->d2, mm->d1, mm->loss};
    for (float* f : fs)
        if (f) cudaFree(f);
    __nv_bfloat16* hs[] = {mm->xb, mm->xT, mm->a1, mm->a1T, mm->a2, mm->a2T, mm->dz3h, mm->dz3T, mm->d2h, mm->d2T,
                           mm->d1T, mm->w1T, mm->w2T, mm->w3T, mm->w2n, mm->w3n};
    for (__nv_bfloat16* h : hs)
        if (h) cudaFree(h);
    if (mm->gerr) cudaFree(mm->gerr);
    if (mm->pack) cudaFree(mm->pack);
    if (mm->derr) cudaFree(mm->derr);
    if (mm->yb) cudaFree(mm->yb);
    if (mm->correct) cudaFree(mm->correct);
    if (mm->s) cudaStreamDestroy(mm->s);
    delete mm;
    return ECMG_OK;
}

int ecmg_mlp_param_count(void) { return NPARAM; }

ecmg_status ecmg_mlp_get_params(ecmg_mlp* mm, float* host_out)
{
    if (!mm || !host_out) return ECMG_ERR_INVALID_ARG;
    cudaStreamSynchronize(mm->s);
    return cudaMemcpy(host_out, mm->p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost) == cudaSuccess ? ECMG_OK
                                                                                                       : ECMG_ERR_CUDA;
}

ecmg_status ecmg_mlp_set_params(ecmg_mlp* mm, const float* host_in)
{
    if (!mm || !host_in) return ECMG_ERR_INVALID_ARG;
    for (int i = 0; i < NPARAM; i++)
        if (!std::isfinite(host_in[i])) return ECMG_ERR_INVALID_ARG;
    cudaStreamSynchronize(mm->s);
    if (cudaMemcpy(mm->p, host_in, sizeof(float) * NPARAM, cudaMemcpyHostToDevice) != cudaSuccess) return ECMG_ERR_CUDA;
    mm->packed = false;
    return ECMG_OK;
}

static ecmg_status ensure_batch(ecmg_mlp* mm, int B)
{
    if (B <= mm->cap) return ECMG_OK;
    float** fs[] = {&mm->z1, &mm->z2, &mm->z3, &mm->dz3, &mm->d2, &mm->d1};
    for (float** f : fs)
        if (*f) { cudaFree(*f); *f = nullptr; }
    __nv_bfloat16** hs[] = {&mm->xb, &mm->xT, &mm->a1, &mm->a1T, &mm->a2, &mm->a2T, &mm->dz3h, &mm->dz3T, &mm->d2h,
                            &mm->d2T, &mm->d1T};
    for (__nv_bfloat16** h : hs)
        if (*h) { cudaFree(*h); *h = nullptr; }
    if (mm->yb) { cudaFree(mm->yb); mm->yb = nullptr; }
    const size_t b = (size_t)B, bt = (size_t)((B + 7) & ~7); /* 16-byte rows of the transposed copies */
    auto fa = [](float** p, size_t n) { return cudaMalloc(p, sizeof(float) * n) == cudaSuccess; };
    auto ha = [](__nv_bfloat16** p, size_t n) { return cudaMalloc(p, 2 * n) == cudaSuccess; };
    bool ok = fa(&mm->z1, b * HID) && fa(&mm->z2, b * HID) && fa(&mm->z3, b * OUT) && fa(&mm->dz3, b * OUT) &&
              fa(&mm->d2, b * HID) && fa(&mm->d1, b * HID) && ha(&mm->xb, b * IN) && ha(&mm->xT, bt * IN) &&
              ha(&mm->a1, b * HID) && ha(&mm->a1T, bt * HID) && ha(&mm->a2, b * HID) && ha(&mm->a2T, bt * HID) &&
              ha(&mm->dz3h, b * OUT) && ha(&mm->dz3T, bt * OUT) && ha(&mm->d2h, b * HID) && ha(&mm->d2T, bt * HID) &&
              ha(&mm->d1T, bt * HID) && cudaMalloc(&mm->yb, sizeof(int) * b) == cudaSuccess;
    if (ok && !mm->w1T)
        ok = ha(&mm->w1T, (size_t)IN * HID) && ha(&mm->w2T, (size_t)HID * HID) && ha(&mm->w3T, (size_t)HID * OUT) &&
             ha(&mm->w2n, (size_t)HID * HID) && ha(&mm->w3n, (size_t)HID * OUT) &&
             cudaMalloc(&mm->gerr, sizeof(int)) == cudaSuccess && cudaMemset(mm->gerr, 0, sizeof(int)) == cudaSuccess;
    /* outside any stream capture: the GEMM kernel's shared memory limit */
    if (ok) ok = cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem) ==
                 cudaSuccess;
    if (!ok) return ECMG_ERR_CUDA;
    mm->cap = B;
    mm->capT = (int)bt;
    return ECMG_OK;
}

/* [rows x cols] BF16 row-major with `ld` elements per row as a 2D tensor;
   boxes of 8 columns x box_rows rows, reads beyond the tensor give zeros */
static cudaError_t bf16_map(CUtensorMap* tm, const void* p, int rows, int cols, int ld, int box_rows)
{
    EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {8, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(p), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

/* C[M x N] (+)= A[M x K] B[N x K]^T on the tensor cores (k_tc_gemm); A has
   lda, B ldb elements per row; split > 1 cuts K over CTAs, added atomically
   into C (which must hold the initial value) */
static cudaError_t tc_gemm(ecmg_mlp* mm, int M, int N, int K, const __nv_bfloat16* A, int lda,
                           const __nv_bfloat16* B, int ldb, float* C, int ldc, int split)
{
    CUtensorMap ta, tb;
    cudaError_t e = bf16_map(&ta, A, M, K, lda, kTile);
    if (e == cudaSuccess) e = bf16_map(&tb, B, N, K, ldb, N);
    if (e != cudaSuccess) return e;
    int kper = (K + split - 1) / split;
    kper = (kper + kGemmKC - 1) / kGemmKC * kGemmKC;
    const dim3 grid((M + kTile - 1) / kTile, (K + kper - 1) / kper);
    k_tc_gemm<<<grid, 128, kGemmSmem, mm->s>>>(ta, tb, M, N, K, kper, C, ldc, split > 1 ? 1 : 0, mm->gerr, mm->spin);
    return cudaGetLastError();
}

/* forward + backward on B rows (gathered by idx, or sampled with seed);
   leaves gradients in mm->g and the summed loss in mm->loss.  Every GEMM
   takes BF16 operands on the tensor cores and accumulates in FP32; the
   elementwise steps and the master weights stay FP32. */
static cudaError_t fwd_bwd(ecmg_mlp* mm, const void* X, const unsigned char* y, int n, int B, unsigned long long seed,
                           const int* idx)
{
    cudaStream_t s = mm->s;
    const float* P = mm->p;
    float* G = mm->g;
    const int T = mm->capT;
    const dim3 pb(32, 8);
    auto pg = [](int rows, int cols) { return dim3((cols + 31) / 32, (rows + 31) / 32); };
    cudaMemsetAsync(mm->loss, 0, sizeof(float), s);
    cudaMemsetAsync(mm->correct, 0, sizeof(int), s);
    k_wconv<<<64, 256, 0, s>>>(P + OW1, IN, HID, mm->w1T, nullptr);
    k_wconv<<<64, 256, 0, s>>>(P + OW2, HID, HID, mm->w2T, mm->w2n);
    k_wconv<<<64, 256, 0, s>>>(P + OW3, HID, OUT, mm->w3T, mm->w3n);
    k_gather<<<B, 96, 0, s>>>((const __nv_bfloat16*)X, y, n, B, seed, idx, mm->xb, mm->yb);
    k_post<__nv_bfloat16><<<pg(B, IN), pb, 0, s>>>(mm->xb, nullptr, nullptr, B, IN, kPostCopy, nullptr, mm->xT, T);
    cudaError_t e;
    /* forward */
    if ((e = tc_gemm(mm, B, HID, IN, mm->xb, IN, mm->w1T, IN, mm->z1, HID, 1)) != cudaSuccess) return e;
    k_post<float><<<pg(B, HID), pb, 0, s>>>(mm->z1, nullptr, P + OB1, B, HID, kPostGelu, mm->a1, mm->a1T, T);
    if ((e = tc_gemm(mm, B, HID, HID, mm->a1, HID, mm->w2T, HID, mm->z2, HID, 1)) != cudaSuccess) return e;
    k_post<float><<<pg(B, HID), pb, 0, s>>>(mm->z2, nullptr, P + OB2, B, HID, kPostGelu, mm->a2, mm->a2T, T);
    if ((e = tc_gemm(mm, B, OUT, HID, mm->a2, HID, mm->w3T, HID, mm->z3, OUT, 1)) != cudaSuccess) return e;
    k_bias_act<<<1024, 256, 0, s>>>(mm->z3, nullptr, P + OB3, B, OUT, 0);
    k_softmax_ce<<<(B + 3) / 4, dim3(32, 4), 0, s>>>(mm->z3, mm->yb, B, mm->dz3, mm->loss, mm->correct);
    k_post<float><<<pg(B, OUT), pb, 0, s>>>(mm->dz3, nullptr, nullptr, B, OUT, kPostCopy, mm->dz3h, mm->dz3T, T);
    /* backward: weight gradients reduce over the batch, split over CTAs */
    const int split = std::max(1, std::min(128, B / 512));
    const int csplit = B >= 4096 ? 256 : 1;
    cudaMemsetAsync(G, 0, sizeof(float) * NPARAM, s);
    if ((e = tc_gemm(mm, HID, OUT, B, mm->a2T, T, mm->dz3T, T, G + OW3, OUT, split)) != cudaSuccess) return e;
    k_colsum<<<dim3((OUT + 127) / 128, csplit), 128, 0, s>>>(mm->dz3, B, OUT, G + OB3);
    if ((e = tc_gemm(mm, B, HID, OUT, mm->dz3h, OUT, mm->w3n, OUT, mm->d2, HID, 1)) != cudaSuccess) return e;
    k_post<float><<<pg(B, HID), pb, 0, s>>>(mm->d2, mm->z2, nullptr, B, HID, kPostBack, mm->d2h, mm->d2T, T);
    if ((e = tc_gemm(mm, HID, HID, B, mm->a1T, T, mm->d2T, T, G + OW2, HID, split)) != cudaSuccess) return e;
    k_colsum<<<dim3((HID + 127) / 128, csplit), 128, 0, s>>>(mm->d2, B, HID, G + OB2);
    if ((e = tc_gemm(mm, B, HID, HID, mm->d2h, HID, mm->w2n, HID, mm->d1, HID, 1)) != cudaSuccess) return e;
    k_post<float><<<pg(B, HID), pb, 0, s>>>(mm->d1, mm->z1, nullptr, B, HID, kPostBack, nullptr, mm->d1T, T);
    if ((e = tc_gemm(mm, IN, HID, B, mm->xT, T, mm->d1T, T, G + OW1, HID, split)) != cudaSuccess) return e;
    k_colsum<<<dim3((HID + 127) / 128, csplit), 128, 0, s>>>(mm->d1, B, HID, G + OB1);
    return cudaGetLastError();
}

/* a tensor-core wait of the training GEMMs timed out (flag cleared) */
static bool gemm_timed_out(ecmg_mlp* mm)
{
    int h = 0;
    if (cudaMemcpyAsync(&h, mm->gerr, sizeof(int), cudaMemcpyDeviceToHost, mm->s) != cudaSuccess ||
        cudaStreamSynchronize(mm->s) != cudaSuccess)
        return true;
    if (h) cudaMemsetAsync(mm->gerr, 0, sizeof(int), mm->s);
    return h != 0;
}

ecmg_status ecmg_mlp_loss_grad(ecmg_mlp* mm, const void* dev_x, const unsigned char* dev_y, int n, float* loss,
                               float* host_grad)
{
    if (!mm || !dev_x || !dev_y || n < 1) return ECMG_ERR_INVALID_ARG;
    if (ensure_batch(mm, n) != ECMG_OK) return ECMG_ERR_CUDA;
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    int* didx = nullptr;
    if (cudaMalloc(&didx, sizeof(int) * n) != cudaSuccess) return ECMG_ERR_CUDA;
    cudaMemcpy(didx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    cudaError_t e = fwd_bwd(mm, dev_x, dev_y, n, n, 0, didx);
    if (e == cudaSuccess) e = cudaStreamSynchronize(mm->s);
    cudaFree(didx);
    if (e != cudaSuccess) return ECMG_ERR_CUDA;
    if (gemm_timed_out(mm)) return ECMG_ERR_BOUND;
    float l = 0;
    cudaMemcpy(&l, mm->loss, sizeof(float), cudaMemcpyDeviceToHost);
    if (loss) *loss = l / (float)n;
    if (host_grad) cudaMemcpy(host_grad, mm->g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
    return ECMG_OK;
}

ecmg_status ecmg_mlp_train(ecmg_mlp* mm, const void* dev_x, const unsigned char* dev_y, int n, int steps, int batch,
                           float lr, unsigned long long seed, float* host_loss, float* host_acc)
{
    if (!mm || !dev_x || !dev_y || n < 1 || steps < 0 || batch < 1 || !(lr > 0.0f)) return ECMG_ERR_INVALID_ARG;
    if (ensure_batch(mm, batch) != ECMG_OK) return ECMG_ERR_CUDA;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < steps; it++) {
        if (fwd_bwd(mm, dev_x, dev_y, n, batch, seed + 0x51ED27ull * (unsigned long long)(mm->step + 1), nullptr) !=
            cudaSuccess)
            return ECMG_ERR_CUDA;
        mm->step++;
        float c1 = 1.0f - powf(b1, (float)mm->step), c2 = 1.0f - powf(b2, (float)mm->step);
        k_adam<<<(NPARAM + 255) / 256, 256, 0, mm->s>>>(mm->p, mm->g, mm->m, mm->v, NPARAM, lr, b1, b2, eps, c1, c2);
        if (host_loss || host_acc) {
            float l = 0;
            int cc = 0;
            cudaMemcpyAsync(&l, mm->loss, sizeof(float), cudaMemcpyDeviceToHost, mm->s);
            cudaMemcpyAsync(&cc, mm->correct, sizeof(int), cudaMemcpyDeviceToHost, mm->s);
            if (cudaStreamSynchronize(mm->s) != cudaSuccess) return ECMG_ERR_CUDA;
            if (host_loss) host_loss[it] = l / (float)batch;
            if (host_acc) host_acc[it] = (float)cc / (float)batch;
        }
    }
    mm->packed = false;
    if (cudaStreamSynchronize(mm->s) != cudaSuccess) return ECMG_ERR_CUDA;
    return gemm_timed_out(mm) ? ECMG_ERR_BOUND : ECMG_OK;
}

ecmg_status ecmg_mlp_set_wait_limit(ecmg_mlp* mm, int polls)
{
    if (!mm || polls < 0) return ECMG_ERR_INVALID_ARG;
    mm->spin = polls > 0 ? polls : kSpinDefault;
    return ECMG_OK;
}

ecmg_status ecmg_mlp_predict(ecmg_mlp* mm, const void* dev_x, int n, unsigned char* dev_cls)
{
    if (!mm || !dev_x || !dev_cls || n < 0) return ECMG_ERR_INVALID_ARG;
    if (n == 0) return ECMG_OK;
    if (ecmg::mlp_pack(mm) != cudaSuccess) return ECMG_ERR_CUDA;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaMemsetAsync(mm->derr, 0, sizeof(int), mm->s) != cudaSuccess) return ECMG_ERR_CUDA;
    if (ecmg::mlp_infer(mm, dev_x, nullptr, n, dev_cls, mm->s, sms, mm->derr, 1) != cudaSuccess) return ECMG_ERR_CUDA;
    int herr = 0;
    if (cudaMemcpyAsync(&herr, mm->derr, sizeof(int), cudaMemcpyDeviceToHost, mm->s) != cudaSuccess ||
        cudaStreamSynchronize(mm->s) != cudaSuccess)
        return ECMG_ERR_CUDA;
    return herr ? ECMG_ERR_BOUND : ECMG_OK;
}

}  // extern "C"
