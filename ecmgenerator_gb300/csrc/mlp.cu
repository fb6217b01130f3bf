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
 * Inference: BF16 weights and activations on the tensor cores
 * (mma.sync m16n8k16, FP32 accumulation), weights staged once per block in
 * shared memory in fragment order.  Training: FP32 master weights, FP32
 * forward/backward GEMMs on the CUDA cores, softmax cross-entropy, Adam.
 * This translation unit is not part of the parity-critical arithmetic.
 */
#include "../../include/ecmg.h"
#include "ecmg_internal.h"

#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <vector>

using namespace ecmg;

namespace {

constexpr int IN = kMlpIn, HID = kMlpHid, OUT = kMlpOut;
constexpr int XS = IN + 8;   /* smem row stride (bf16) of an input tile: conflict-free fragment loads */
constexpr int HS = HID + 8;  /* smem row stride of a hidden tile */
constexpr int W1F = (IN / 16) * (HID / 8) * 64;   /* u32 words of packed layer-1 fragments */
constexpr int W2F = (HID / 16) * (HID / 8) * 64;
constexpr int W3F = (HID / 16) * (OUT / 8) * 64;

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

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

/* W is [K x N] row-major FP32; packed as B fragments of m16n8k16:
   word ((ks * (N/8) + nt) * 32 + lane) * 2 + r holds rows
   ks*16 + (lane%4)*2 + 8r + {0,1} of column nt*8 + lane/4 */
__global__ void k_pack_b(const float* W, int K, int N, uint32_t* out)
{
    int total = (K / 16) * (N / 8) * 64;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        int r = i & 1, lane = (i >> 1) & 31, f = i >> 6;
        int nt = f % (N / 8), ks = f / (N / 8);
        int k = ks * 16 + (lane & 3) * 2 + 8 * r;
        int n = nt * 8 + (lane >> 2);
        out[i] = pack_bf16(W[(size_t)k * N + n], W[(size_t)(k + 1) * N + n]);
    }
}

/* A fragment of rows [r0, r0+16) from a bf16 smem tile with row stride `s` */
__device__ __forceinline__ void load_a(const __nv_bfloat16* t, int s, int ks, int lane, uint32_t* a)
{
    int g = lane >> 2, c = ks * 16 + (lane & 3) * 2;
    const uint32_t* p0 = reinterpret_cast<const uint32_t*>(t + g * s + c);
    const uint32_t* p1 = reinterpret_cast<const uint32_t*>(t + (g + 8) * s + c);
    a[0] = p0[0];
    a[1] = p1[0];
    a[2] = p0[4]; /* +8 columns */
    a[3] = p1[4];
}

/* One warp: 16 rows through the three layers.  xin: 16 x XS bf16 tile in
   smem; hbuf: 16 x HS bf16 scratch; returns per-row argmax in lanes
   (lane/4 -> row lane/4, row lane/4 + 8). */
__device__ void mlp_tile(const __nv_bfloat16* xin, __nv_bfloat16* hbuf, const uint32_t* w1, const uint32_t* w2,
                         const uint32_t* w3, const float* b1, const float* b2, const float* b3, int lane,
                         int* cls_lo, int* cls_hi)
{
    const int g = lane >> 2, tg = lane & 3;
    float acc[OUT / 8][4];
    /* layer 1 */
#pragma unroll
    for (int nt = 0; nt < HID / 8; nt++) {
        float bb0 = b1[nt * 8 + tg * 2], bb1 = b1[nt * 8 + tg * 2 + 1];
        acc[nt][0] = bb0; acc[nt][1] = bb1; acc[nt][2] = bb0; acc[nt][3] = bb1;
    }
#pragma unroll
    for (int ks = 0; ks < IN / 16; ks++) {
        uint32_t a[4];
        load_a(xin, XS, ks, lane, a);
#pragma unroll
        for (int nt = 0; nt < HID / 8; nt++) {
            const uint2 b = reinterpret_cast<const uint2*>(w1)[(ks * (HID / 8) + nt) * 32 + lane];
            uint32_t bb[2] = {b.x, b.y};
            mma_bf16(acc[nt], a, bb);
        }
    }
#pragma unroll
    for (int nt = 0; nt < HID / 8; nt++) {
        int c = nt * 8 + tg * 2;
        *reinterpret_cast<uint32_t*>(hbuf + g * HS + c) = pack_bf16(gelu(acc[nt][0]), gelu(acc[nt][1]));
        *reinterpret_cast<uint32_t*>(hbuf + (g + 8) * HS + c) = pack_bf16(gelu(acc[nt][2]), gelu(acc[nt][3]));
    }
    __syncwarp();
    /* layer 2 */
#pragma unroll
    for (int nt = 0; nt < HID / 8; nt++) {
        float bb0 = b2[nt * 8 + tg * 2], bb1 = b2[nt * 8 + tg * 2 + 1];
        acc[nt][0] = bb0; acc[nt][1] = bb1; acc[nt][2] = bb0; acc[nt][3] = bb1;
    }
#pragma unroll
    for (int ks = 0; ks < HID / 16; ks++) {
        uint32_t a[4];
        load_a(hbuf, HS, ks, lane, a);
#pragma unroll
        for (int nt = 0; nt < HID / 8; nt++) {
            const uint2 b = reinterpret_cast<const uint2*>(w2)[(ks * (HID / 8) + nt) * 32 + lane];
            uint32_t bb[2] = {b.x, b.y};
            mma_bf16(acc[nt], a, bb);
        }
    }
    __syncwarp();
#pragma unroll
    for (int nt = 0; nt < HID / 8; nt++) {
        int c = nt * 8 + tg * 2;
        *reinterpret_cast<uint32_t*>(hbuf + g * HS + c) = pack_bf16(gelu(acc[nt][0]), gelu(acc[nt][1]));
        *reinterpret_cast<uint32_t*>(hbuf + (g + 8) * HS + c) = pack_bf16(gelu(acc[nt][2]), gelu(acc[nt][3]));
    }
    __syncwarp();
    /* layer 3 */
#pragma unroll
    for (int nt = 0; nt < OUT / 8; nt++) {
        float bb0 = b3[nt * 8 + tg * 2], bb1 = b3[nt * 8 + tg * 2 + 1];
        acc[nt][0] = bb0; acc[nt][1] = bb1; acc[nt][2] = bb0; acc[nt][3] = bb1;
    }
#pragma unroll
    for (int ks = 0; ks < HID / 16; ks++) {
        uint32_t a[4];
        load_a(hbuf, HS, ks, lane, a);
#pragma unroll
        for (int nt = 0; nt < OUT / 8; nt++) {
            const uint2 b = reinterpret_cast<const uint2*>(w3)[(ks * (OUT / 8) + nt) * 32 + lane];
            uint32_t bb[2] = {b.x, b.y};
            mma_bf16(acc[nt], a, bb);
        }
    }
    /* argmax of rows g and g+8 over this lane's columns, then across the 4
       lanes sharing the row (ties: the lower class) */
    float v0 = -INFINITY, v1 = -INFINITY;
    int i0 = 0, i1 = 0;
#pragma unroll
    for (int nt = 0; nt < OUT / 8; nt++) {
#pragma unroll
        for (int e = 0; e < 2; e++) {
            int c = nt * 8 + tg * 2 + e;
            if (acc[nt][e] > v0) { v0 = acc[nt][e]; i0 = c; }
            if (acc[nt][2 + e] > v1) { v1 = acc[nt][2 + e]; i1 = c; }
        }
    }
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) {
        float ov0 = __shfl_xor_sync(0xffffffffu, v0, o), ov1 = __shfl_xor_sync(0xffffffffu, v1, o);
        int oi0 = __shfl_xor_sync(0xffffffffu, i0, o), oi1 = __shfl_xor_sync(0xffffffffu, i1, o);
        if (ov0 > v0 || (ov0 == v0 && oi0 < i0)) { v0 = ov0; i0 = oi0; }
        if (ov1 > v1 || (ov1 == v1 && oi1 < i1)) { v1 = ov1; i1 = oi1; }
    }
    *cls_lo = i0;
    *cls_hi = i1;
}

constexpr int kInferWarps = 8;
constexpr size_t kInferSmem = sizeof(uint32_t) * (W1F + W2F + W3F) + sizeof(float) * (2 * HID + OUT) +
                              (size_t)kInferWarps * sizeof(__nv_bfloat16) * (16 * XS + 16 * HS);

/* class of every row of X [n, IN] (bf16, row-major) */
__global__ void __launch_bounds__(32 * kInferWarps) k_mlp_infer(const __nv_bfloat16* X, const int* n_ptr, int n_fixed,
                                                                const uint32_t* wpack, const float* bias,
                                                                unsigned char* cls)
{
    extern __shared__ __align__(16) unsigned char sm[];
    uint32_t* w = reinterpret_cast<uint32_t*>(sm);
    float* bs = reinterpret_cast<float*>(w + W1F + W2F + W3F);
    __nv_bfloat16* tiles = reinterpret_cast<__nv_bfloat16*>(bs + 2 * HID + OUT);
    const int n = n_ptr ? *n_ptr : n_fixed;
    /* weights and biases, once per block */
    for (int i = threadIdx.x; i < (W1F + W2F + W3F) / 4; i += blockDim.x)
        reinterpret_cast<uint4*>(w)[i] = reinterpret_cast<const uint4*>(wpack)[i];
    for (int i = threadIdx.x; i < 2 * HID + OUT; i += blockDim.x) bs[i] = bias[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16* xt = tiles + warp * (16 * XS + 16 * HS);
    __nv_bfloat16* ht = xt + 16 * XS;
    const int ntile = (n + 15) / 16;
    for (int tile = blockIdx.x * kInferWarps + warp; tile < ntile; tile += gridDim.x * kInferWarps) {
        int r0 = tile * 16;
        /* 16 rows x 96 bf16 = 16 x 12 uint4 */
        for (int i = lane; i < 16 * (IN / 8); i += 32) {
            int rr = i / (IN / 8), cc = i % (IN / 8);
            uint4 v = make_uint4(0, 0, 0, 0);
            if (r0 + rr < n) v = reinterpret_cast<const uint4*>(X + (size_t)(r0 + rr) * IN)[cc];
            *reinterpret_cast<uint4*>(xt + rr * XS + cc * 8) = v;
        }
        __syncwarp();
        int c0, c1;
        mlp_tile(xt, ht, w, w + W1F, w + W1F + W2F, bs, bs + HID, bs + 2 * HID, lane, &c0, &c1);
        if ((lane & 3) == 0) {
            int g = lane >> 2;
            if (r0 + g < n) cls[r0 + g] = (unsigned char)c0;
            if (r0 + g + 8 < n) cls[r0 + g + 8] = (unsigned char)c1;
        }
        __syncwarp();
    }
}

/* ------------------------------------------------------------------------
 * Training (FP32 on the CUDA cores)
 * ---------------------------------------------------------------------- */

/* C[M x N] (+)= op(A)[M x K] * op(B)[K x N]; row-major storage, lda/ldb/ldc
   are row strides of the stored matrices.  With split > 1 the K range is cut
   into `split` parts accumulated atomically (C must hold the initial value). */
template <bool TA, bool TB>
__global__ void k_gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                       int split, int accumulate)
{
    __shared__ float sa[32][33], sb[32][33];
    int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5; /* 32 x 8 threads, 4 rows each */
    int kchunk = (K + split - 1) / split;
    int k0 = bz * kchunk, k1 = min(K, k0 + kchunk);
    float acc[4] = {0, 0, 0, 0};
    for (int kk = k0; kk < k1; kk += 32) {
        /* sa[m][k], sb[k][n]; consecutive threads read consecutive addresses */
        for (int r = ty; r < 32; r += 8) {
            if (TA) {
                int m = by * 32 + tx, k = kk + r;
                sa[tx][r] = (m < M && k < k1) ? A[(size_t)k * lda + m] : 0.0f;
            } else {
                int m = by * 32 + r, k = kk + tx;
                sa[r][tx] = (m < M && k < k1) ? A[(size_t)m * lda + k] : 0.0f;
            }
            if (TB) {
                int nb = bx * 32 + r, kb = kk + tx;
                sb[tx][r] = (kb < k1 && nb < N) ? B[(size_t)nb * ldb + kb] : 0.0f;
            } else {
                int kb = kk + r, nb = bx * 32 + tx;
                sb[r][tx] = (kb < k1 && nb < N) ? B[(size_t)kb * ldb + nb] : 0.0f;
            }
        }
        __syncthreads();
#pragma unroll 8
        for (int q = 0; q < 32; q++) {
            float b = sb[q][tx];
#pragma unroll
            for (int i = 0; i < 4; i++) acc[i] += sa[ty + 8 * i][q] * b;
        }
        __syncthreads();
    }
    for (int i = 0; i < 4; i++) {
        int m = by * 32 + ty + 8 * i, nn = bx * 32 + tx;
        if (m < M && nn < N) {
            float* c = C + (size_t)m * ldc + nn;
            if (split > 1) atomicAdd(c, acc[i]);
            else *c = accumulate ? *c + acc[i] : acc[i];
        }
    }
}

template <bool TA, bool TB>
static void gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc, int split,
                 int accumulate, cudaStream_t s)
{
    dim3 grid((N + 31) / 32, (M + 31) / 32, split);
    k_gemm<TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, split, accumulate);
}

__global__ void k_gather(const __nv_bfloat16* X, const unsigned char* y, int n, int B, unsigned long long seed,
                         const int* idx, float* xb, int* yb)
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
    for (int c = threadIdx.x; c < IN; c += blockDim.x) xb[(size_t)r * IN + c] = __bfloat162float(X[(size_t)src * IN + c]);
    if (threadIdx.x == 0) yb[r] = y[src];
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

__global__ void k_gelu_back(float* dA, const float* Z, size_t total)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        dA[i] *= gelu_grad(Z[i]);
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
    uint32_t* pack = nullptr; /* BF16 fragment-packed weights for inference */
    float* bias = nullptr;  /* b1 | b2 | b3 */
    int step = 0;
    bool packed = false;
    /* training scratch for batch B */
    int cap = 0;
    float *xb = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr, *z3 = nullptr, *dz3 = nullptr,
          *d2 = nullptr, *d1 = nullptr, *loss = nullptr;
    int *yb = nullptr, *correct = nullptr;
    cudaStream_t s = nullptr;
};

namespace ecmg {
/* used by the tick (ctx.cu) */
cudaError_t mlp_infer(ecmg_mlp* mlp, const void* X, const int* n_dev, int n_max, unsigned char* cls, cudaStream_t s,
                      int sms);
cudaError_t mlp_pack(ecmg_mlp* mlp);
}  // namespace ecmg

cudaError_t ecmg::mlp_pack(ecmg_mlp* mm)
{
    /* outside any stream capture: the inference kernel's shared memory limit */
    cudaError_t ea = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
    if (ea != cudaSuccess) return ea;
    if (mm->packed) return cudaSuccess;
    k_pack_b<<<64, 256, 0, mm->s>>>(mm->p + OW1, IN, HID, mm->pack);
    k_pack_b<<<64, 256, 0, mm->s>>>(mm->p + OW2, HID, HID, mm->pack + W1F);
    k_pack_b<<<64, 256, 0, mm->s>>>(mm->p + OW3, HID, OUT, mm->pack + W1F + W2F);
    cudaMemcpyAsync(mm->bias, mm->p + OB1, sizeof(float) * HID, cudaMemcpyDeviceToDevice, mm->s);
    cudaMemcpyAsync(mm->bias + HID, mm->p + OB2, sizeof(float) * HID, cudaMemcpyDeviceToDevice, mm->s);
    cudaMemcpyAsync(mm->bias + 2 * HID, mm->p + OB3, sizeof(float) * OUT, cudaMemcpyDeviceToDevice, mm->s);
    cudaError_t e = cudaStreamSynchronize(mm->s);
    if (e == cudaSuccess) mm->packed = true;
    return e;
}

cudaError_t ecmg::mlp_infer(ecmg_mlp* mm, const void* X, const int* n_dev, int n_max, unsigned char* cls,
                            cudaStream_t s, int sms)
{
    int tiles = (n_max + 15) / 16;
    int grid = (tiles + kInferWarps - 1) / kInferWarps;
    if (grid > sms) grid = sms; /* one block per SM holds the weights once */
    if (grid < 1) grid = 1;
    k_mlp_infer<<<grid, 32 * kInferWarps, kInferSmem, s>>>((const __nv_bfloat16*)X, n_dev, n_max, mm->pack, mm->bias,
                                                           cls);
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
              cudaMalloc(&mm->pack, sizeof(uint32_t) * (W1F + W2F + W3F)) == cudaSuccess &&
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
    float* fs[] = {mm->p, mm->g, mm->m, mm->v, mm->bias, mm->xb, mm->z1, mm->a1, mm->z2, mm->a2, mm->z3, mm->dz3,
                   mm->d2, mm->d1, mm->loss};
    for (float* f : fs)
        if (f) cudaFree(f);
    if (mm->pack) cudaFree(mm->pack);
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
    float** fs[] = {&mm->xb, &mm->z1, &mm->a1, &mm->z2, &mm->a2, &mm->z3, &mm->dz3, &mm->d2, &mm->d1};
    for (float** f : fs)
        if (*f) { cudaFree(*f); *f = nullptr; }
    if (mm->yb) { cudaFree(mm->yb); mm->yb = nullptr; }
    size_t b = (size_t)B;
    bool ok = cudaMalloc(&mm->xb, sizeof(float) * b * IN) == cudaSuccess &&
              cudaMalloc(&mm->z1, sizeof(float) * b * HID) == cudaSuccess &&
              cudaMalloc(&mm->a1, sizeof(float) * b * HID) == cudaSuccess &&
              cudaMalloc(&mm->z2, sizeof(float) * b * HID) == cudaSuccess &&
              cudaMalloc(&mm->a2, sizeof(float) * b * HID) == cudaSuccess &&
              cudaMalloc(&mm->z3, sizeof(float) * b * OUT) == cudaSuccess &&
              cudaMalloc(&mm->dz3, sizeof(float) * b * OUT) == cudaSuccess &&
              cudaMalloc(&mm->d2, sizeof(float) * b * HID) == cudaSuccess &&
              cudaMalloc(&mm->d1, sizeof(float) * b * HID) == cudaSuccess &&
              cudaMalloc(&mm->yb, sizeof(int) * b) == cudaSuccess;
    if (!ok) return ECMG_ERR_CUDA;
    mm->cap = B;
    return ECMG_OK;
}

/* forward + backward on B rows (gathered by idx, or sampled with seed);
   leaves gradients in mm->g and the summed loss in mm->loss */
static void fwd_bwd(ecmg_mlp* mm, const void* X, const unsigned char* y, int n, int B, unsigned long long seed,
                    const int* idx)
{
    cudaStream_t s = mm->s;
    const float* P = mm->p;
    float* G = mm->g;
    cudaMemsetAsync(mm->loss, 0, sizeof(float), s);
    cudaMemsetAsync(mm->correct, 0, sizeof(int), s);
    k_gather<<<B, 96, 0, s>>>((const __nv_bfloat16*)X, y, n, B, seed, idx, mm->xb, mm->yb);
    gemm<false, false>(B, HID, IN, mm->xb, IN, P + OW1, HID, mm->z1, HID, 1, 0, s);
    k_bias_act<<<1024, 256, 0, s>>>(mm->z1, mm->a1, P + OB1, B, HID, 1);
    gemm<false, false>(B, HID, HID, mm->a1, HID, P + OW2, HID, mm->z2, HID, 1, 0, s);
    k_bias_act<<<1024, 256, 0, s>>>(mm->z2, mm->a2, P + OB2, B, HID, 1);
    gemm<false, false>(B, OUT, HID, mm->a2, HID, P + OW3, OUT, mm->z3, OUT, 1, 0, s);
    k_bias_act<<<1024, 256, 0, s>>>(mm->z3, nullptr, P + OB3, B, OUT, 0);
    k_softmax_ce<<<(B + 3) / 4, dim3(32, 4), 0, s>>>(mm->z3, mm->yb, B, mm->dz3, mm->loss, mm->correct);
    int split = B >= 4096 ? 32 : 1;
    int csplit = B >= 4096 ? 256 : 1;
    cudaMemsetAsync(G, 0, sizeof(float) * NPARAM, s);
    /* layer 3 */
    gemm<true, false>(HID, OUT, B, mm->a2, HID, mm->dz3, OUT, G + OW3, OUT, split, 0, s);
    k_colsum<<<dim3((OUT + 127) / 128, csplit), 128, 0, s>>>(mm->dz3, B, OUT, G + OB3);
    gemm<false, true>(B, HID, OUT, mm->dz3, OUT, P + OW3, OUT, mm->d2, HID, 1, 0, s);
    k_gelu_back<<<1024, 256, 0, s>>>(mm->d2, mm->z2, (size_t)B * HID);
    /* layer 2 */
    gemm<true, false>(HID, HID, B, mm->a1, HID, mm->d2, HID, G + OW2, HID, split, 0, s);
    k_colsum<<<dim3((HID + 127) / 128, csplit), 128, 0, s>>>(mm->d2, B, HID, G + OB2);
    gemm<false, true>(B, HID, HID, mm->d2, HID, P + OW2, HID, mm->d1, HID, 1, 0, s);
    k_gelu_back<<<1024, 256, 0, s>>>(mm->d1, mm->z1, (size_t)B * HID);
    /* layer 1 */
    gemm<true, false>(IN, HID, B, mm->xb, IN, mm->d1, HID, G + OW1, HID, split, 0, s);
    k_colsum<<<dim3((HID + 127) / 128, csplit), 128, 0, s>>>(mm->d1, B, HID, G + OB1);
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
    fwd_bwd(mm, dev_x, dev_y, n, n, 0, didx);
    cudaError_t e = cudaStreamSynchronize(mm->s);
    cudaFree(didx);
    if (e != cudaSuccess) return ECMG_ERR_CUDA;
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
        fwd_bwd(mm, dev_x, dev_y, n, batch, seed + 0x51ED27ull * (unsigned long long)(mm->step + 1), nullptr);
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
    return cudaStreamSynchronize(mm->s) == cudaSuccess ? ECMG_OK : ECMG_ERR_CUDA;
}

ecmg_status ecmg_mlp_predict(ecmg_mlp* mm, const void* dev_x, int n, unsigned char* dev_cls)
{
    if (!mm || !dev_x || !dev_cls || n < 0) return ECMG_ERR_INVALID_ARG;
    if (n == 0) return ECMG_OK;
    if (ecmg::mlp_pack(mm) != cudaSuccess) return ECMG_ERR_CUDA;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ecmg::mlp_infer(mm, dev_x, nullptr, n, dev_cls, mm->s, sms) != cudaSuccess) return ECMG_ERR_CUDA;
    return cudaStreamSynchronize(mm->s) == cudaSuccess ? ECMG_OK : ECMG_ERR_CUDA;
}

}  // extern "C"
