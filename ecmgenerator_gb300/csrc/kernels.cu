/*
 * kernels.cu -- the per-tick kernels.
 *
 * One tick (Simulator::Update, ECMAgentSimulator/Simulator.cpp:314-323) is
 *   k_bin      bucket every active slot into the uniform agent grid
 *   k_scan_*   exclusive scan of the bucket counts
 *   k_scatter  tick-start snapshot of position/velocity/radius in grid order
 *   k_attract  attraction point (IRM) and preferred velocity (second stream)
 *   k_neighbors exact kNN on the grid
 *   k_agents   one thread per agent: obstacle + agent ORCA half-planes,
 *              2D LP (+3D LP), velocity and position update
 *              (k_agents_warp: one warp per agent; k_agents_knn: the kNN and
 *              the step in one persistent kernel)
 * The snapshot makes the tick Jacobi-exact: neighbours are read from the
 * tick-start copy while each thread writes its own slot, which is what the
 * reference's system order guarantees (velocities change only in
 * UpdateVelocitySystem, after every agent's ORCA query).
 *
 * Built with -fmad=false: every float expression is the reference's sequence
 * of separately rounded operations.
 */
#include "ecmg_internal.h"

#include <cuda_bf16.h>
#include <stdint.h>

namespace ecmg {

/* ---------------------------------------------------------------------- */
/* grid cell of a position; cells outside [0,gw)x[0,gh) -> overflow bucket  */
__device__ __forceinline__ void cell_of(const AgentGrid& g, V2 p, int* cx, int* cy)
{
    float fx = (p.x - g.x0) * g.inv;
    float fy = (p.y - g.y0) * g.inv;
    fx = fminf(fmaxf(fx, -1.0e6f), 1.0e6f); /* NaN -> -1e6 (fmaxf drops NaN) */
    fy = fminf(fmaxf(fy, -1.0e6f), 1.0e6f);
    *cx = (int)floorf(fx);
    *cy = (int)floorf(fy);
}

__device__ __forceinline__ int bucket_of(const AgentGrid& g, V2 p)
{
    int cx, cy;
    cell_of(g, p, &cx, &cy);
    if (cx < 0 || cy < 0 || cx >= g.gw || cy >= g.gh) return g.ncells;
    return cy * g.gw + cx;
}

__global__ void k_bin(BinArgs a)
{
    const int last = a.n_fixed > 0 ? a.n_fixed - 1 : a.counters[C_LAST];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= last; i += gridDim.x * blockDim.x) {
        if (!a.active[i]) continue;
        int b;
        if (a.scenes) {
            const SceneDev& sc = a.scenes[a.slot_scene ? a.slot_scene[i] : 0];
            b = sc.bucket_base + bucket_of(sc.grid, a.pos[i]);
        } else {
            b = bucket_of(a.grid, a.pos[i]);
        }
        a.key[i] = b;
        a.rank[i] = atomicAdd(&a.cell_count[b], 1);
    }
}

__global__ void k_scatter(BinArgs a)
{
    const int last = a.n_fixed > 0 ? a.n_fixed - 1 : a.counters[C_LAST];
    if (blockIdx.x == 0 && threadIdx.x == 0) a.counters[C_NSORTED] = a.cell_start[a.total_buckets];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= last; i += gridDim.x * blockDim.x) {
        if (!a.active[i]) continue;
        int d = a.cell_start[a.key[i]] + a.rank[i];
        a.s_slot[d] = i;
        a.s_pos[d] = a.pos[i];
        if (a.s_vel) a.s_vel[d] = a.vel[i];
        if (a.s_clear) a.s_clear[d] = a.clear[i];
    }
}

/* ---- exclusive scan of n ints (n <= 1024 * 1024 * 4 per pass) ------------ */
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh, int* total)
{
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < (blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    int incl = x + (w > 0 ? sh[w - 1] : 0);
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return incl - v;
}

__global__ void k_scan_local(const int* in, int* out, int* block_sums, int n)
{
    __shared__ int sh[32];
    int i = blockIdx.x * kScanBlock + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int tot;
    int ex = block_exclusive_scan(v, sh, &tot);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void k_scan_top(int* block_sums, int nb, int* out, int n)
{
    __shared__ int sh[32];
    int carry = 0;
    for (int base = 0; base < nb; base += kScanBlock) {
        int i = base + threadIdx.x;
        int v = i < nb ? block_sums[i] : 0;
        int tot;
        int ex = block_exclusive_scan(v, sh, &tot);
        if (i < nb) block_sums[i] = ex + carry;
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry; /* total after the last element */
}

__global__ void k_scan_add(int* out, const int* block_sums, int n)
{
    int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

int scan_tmp_ints(int n) { return (n + kScanBlock - 1) / kScanBlock + 32; }

/* out[0..n] = exclusive scan of in[0..n-1], out[n] = total */
static cudaError_t scan(const int* in, int* out, int n, int* tmp, cudaStream_t s)
{
    int nb = (n + kScanBlock - 1) / kScanBlock;
    k_scan_local<<<nb, kScanBlock, 0, s>>>(in, out, tmp, n);
    k_scan_top<<<1, kScanBlock, 0, s>>>(tmp, nb, out, n);
    k_scan_add<<<nb, kScanBlock, 0, s>>>(out, tmp, n);
    return cudaGetLastError();
}

/* ---------------------------------------------------------------------- */
/* exact kNN on the grid: the k smallest (d2, slot) with EPS < d2 < r^2.
   keys: d2 bits (non-negative floats order as unsigned ints) : slot.
   The list holds the k nearest in key[K-k .. K-1], ascending; key[0 .. K-k)
   hold 0 (below every real key, as d2 > EPS) and never move, unfilled
   entries hold ~0 (above every real key), so the k-th key is key[K-1].  The
   slot in the low half of a key identifies the neighbour; its grid-order
   index is recovered once at the end (bucket start + rank of the slot). */
template <int K>
struct Knn {
    unsigned long long key[K];
    int cnt;
};

template <int K>
__device__ __forceinline__ void knn_consider(Knn<K>& s, int k, int j, V2 p, const V2* s_pos, const int* s_slot,
                                             float r2)
{
    V2 q = s_pos[j];
    float dx = q.x - p.x, dy = q.y - p.y;
    float d2 = dx * dx + dy * dy; /* KDTree.cpp:107-108 */
    if (!(d2 > kEps) || !(d2 < r2)) return;
    unsigned hi = __float_as_uint(d2);
    if (hi > (unsigned)(s.key[K - 1] >> 32)) return;
    unsigned long long kk = ((unsigned long long)hi << 32) | (unsigned)s_slot[j];
    if (kk >= s.key[K - 1]) return;
    /* drop key[K-1], shift the larger entries up, place kk */
#pragma unroll
    for (int q = K - 1; q >= 0; q--) {
        unsigned long long nk;
        if (q > 0 && s.key[q - 1] > kk) nk = s.key[q - 1];
        else if (s.key[q] > kk) nk = kk;
        else nk = s.key[q];
        s.key[q] = nk;
    }
    if (s.cnt < k) s.cnt++;
}

template <int K>
__device__ void knn_grid(Knn<K>& s, int k, V2 p, float rnb, float r2, const V2* s_pos, const int* s_slot,
                         const int* cell_start, const AgentGrid& g)
{
#pragma unroll
    for (int q = 0; q < K; q++) s.key[q] = q < K - k ? 0ull : ~0ull;
    s.cnt = 0;
    int cx, cy;
    cell_of(g, p, &cx, &cy);
    float x0 = g.x0 + (float)cx * g.cell, y0 = g.y0 + (float)cy * g.cell;
    float m = fminf(fminf(p.x - x0, x0 + g.cell - p.x), fminf(p.y - y0, y0 + g.cell - p.y));
    m = fmaxf(m, 0.0f);
    const int rmax = (int)ceilf(rnb * g.inv) + 2;
    /* ring R = -1 is the overflow bucket (agents outside the grid rectangle);
       ring R >= 0 are the cells at Chebyshev distance R.  Every candidate range
       funnels into one loop so that the insertion code exists once. */
    for (int R = -1; R <= rmax; R++) {
        if (R >= 1) {
            /* lower bound of the distance to any agent in ring R or beyond;
               1 cm absorbs the rounding of the bucket assignment */
            float lb = (float)(R - 1) * g.cell + m - 0.01f;
            if (lb >= rnb) break;
            if (s.cnt == k && lb > 0.0f && lb * lb > __uint_as_float((unsigned)(s.key[K - 1] >> 32))) break;
        }
        const int ylo = R < 0 ? 0 : cy - R, yhi = R < 0 ? 0 : cy + R;
        for (int y = ylo; y <= yhi; y++) {
            /* cells whose distance from p (less 1 cm for the rounding of the
               bucket assignment) exceeds the current k-th distance, or the
               neighbour distance, cannot hold an accepted candidate */
            const float kd2 = s.cnt == k ? __uint_as_float((unsigned)(s.key[K - 1] >> 32)) : r2;
            float dy = 0.0f;
            if (R >= 0) {
                const float ry0 = g.y0 + (float)y * g.cell;
                dy = fmaxf(fmaxf(ry0 - p.y, p.y - (ry0 + g.cell)) - 0.01f, 0.0f);
                if (dy * dy > kd2) continue;
            }
            for (int side = 0; side < 2; side++) {
                int j0 = 0, j1 = 0;
                if (R < 0) {
                    if (side == 0) { j0 = cell_start[g.ncells]; j1 = cell_start[g.ncells + 1]; }
                } else if (y >= 0 && y < g.gh) {
                    const int xa = cx - R, xb = cx + R;
                    if (y == ylo || y == yhi) {
                        const float dxm = sqrtf(kd2 - dy * dy) + 0.01f;
                        const int xl = (int)floorf(fmaxf((p.x - dxm - g.x0) * g.inv, -1.0e6f));
                        const int xr = (int)floorf(fminf((p.x + dxm - g.x0) * g.inv, 1.0e6f));
                        int a = max(max(xa, 0), xl), b = min(min(xb, g.gw - 1), xr);
                        if (side == 0 && a <= b) { j0 = cell_start[y * g.gw + a]; j1 = cell_start[y * g.gw + b + 1]; }
                    } else {
                        int x = side == 0 ? xa : xb;
                        if (x >= 0 && x < g.gw && (side == 0 || xb != xa)) {
                            const float rx0 = g.x0 + (float)x * g.cell;
                            const float dx = fmaxf(fmaxf(rx0 - p.x, p.x - (rx0 + g.cell)) - 0.01f, 0.0f);
                            if (!(dx * dx + dy * dy > kd2)) {
                                j0 = cell_start[y * g.gw + x];
                                j1 = cell_start[y * g.gw + x + 1];
                            }
                        }
                    }
                }
                for (int j = j0; j < j1; j++) knn_consider<K>(s, k, j, p, s_pos, s_slot, r2);
            }
        }
    }
}

/* ---------------------------------------------------------------------- */
/* Fast path of the exact kNN: cells in ascending order of their distance.
   The grid cells around an agent's cell (Chebyshev radius <= kTmplR) are
   visited in ascending order of their smallest distance from the quarter of
   the agent's cell that holds the agent (a table built at compile time for
   the lower-left quarter and mirrored for the others), so the k nearest are
   met early and few candidates enter the list only to be dropped again; the
   walk stops at the first cell whose distance bound exceeds the current k-th
   distance.
   The list holds packed keys: a candidate's d2 with its 12 low mantissa bits
   replaced by a code of where it came from (table step, offset in its
   cell), so that one float min / max pair per list position inserts it --
   the ALU pipe's work -- and the code gives its grid index back at the end.
   Packed keys order candidates by d2 except within a relative 2^-11 of each
   other ("near ties"); those groups are re-sorted by the exact (d2, slot)
   key afterwards.  The list keeps two entries beyond the k-th so that a near
   tie at the k-th is resolved inside the list; when it may reach beyond it
   (a dropped candidate with the same leading bits), when a cell holds more
   than 32 agents, when the table ends before the search could (sparse
   crowds) or when the agent is outside the grid, the search returns false
   and the caller runs the 64-bit (d2, slot) search (knn_grid). */
constexpr int kTmplR = 5;
/* bound per axis from the quarter [0, 1/2] of cell 0 to cell d, in half cells */
constexpr int tmpl_half(int d) { return d >= 1 ? 2 * d - 1 : (d <= -1 ? 2 * (-d - 1) : 0); }
/* the table holds the cells whose bound is at most kTmplR cells: every cell
   outside it is at least kTmplR cells away, so a walk that stops inside the
   table has passed every cell that can hold a closer agent */
constexpr bool tmpl_in(int dx, int dy)
{
    return tmpl_half(dx) * tmpl_half(dx) + tmpl_half(dy) * tmpl_half(dy) <= 4 * kTmplR * kTmplR;
}
constexpr int tmpl_count()
{
    int n = 0;
    for (int dy = -kTmplR; dy <= kTmplR; dy++)
        for (int dx = -kTmplR; dx <= kTmplR; dx++) n += tmpl_in(dx, dy) ? 1 : 0;
    return n;
}
constexpr int kTmplN = tmpl_count();
struct KnnTemplate {
    signed char dx[kTmplN], dy[kTmplN];
    unsigned char hx[kTmplN], hy[kTmplN]; /* distance bound per axis in half cells */
};
constexpr KnnTemplate make_knn_template()
{
    KnnTemplate t{};
    int key[kTmplN] = {};
    int n = 0;
    for (int dy = -kTmplR; dy <= kTmplR; dy++)
        for (int dx = -kTmplR; dx <= kTmplR; dx++) {
            if (!tmpl_in(dx, dy)) continue;
            const int hx = tmpl_half(dx), hy = tmpl_half(dy);
            /* squared bound, then the nearer cells first among equal bounds */
            const int kk = (hx * hx + hy * hy) * 1024 + (dx < 0 ? -dx : dx) + (dy < 0 ? -dy : dy);
            int i = n++;
            while (i > 0 && key[i - 1] > kk) {
                key[i] = key[i - 1];
                t.dx[i] = t.dx[i - 1];
                t.dy[i] = t.dy[i - 1];
                t.hx[i] = t.hx[i - 1];
                t.hy[i] = t.hy[i - 1];
                i--;
            }
            key[i] = kk;
            t.dx[i] = (signed char)dx;
            t.dy[i] = (signed char)dy;
            t.hx[i] = (unsigned char)hx;
            t.hy[i] = (unsigned char)hy;
        }
    return t;
}
__constant__ KnnTemplate c_knn_tmpl = make_knn_template();

constexpr unsigned kCodeMask = 0xFFFu;  /* low mantissa bits of a packed key */
constexpr int kCodeOverflow = 127;       /* table step code of the overflow bucket */
static_assert(kTmplN < kCodeOverflow, "table steps must fit 7 bits");

__device__ __forceinline__ unsigned key_hi(float k) { return __float_as_uint(k) & ~kCodeMask; }

/* one candidate (grid index j) into the packed list of KL entries; code =
   table step << 5 | offset in the cell; a candidate not kept, or the entry
   pushed out, lowers *rej */
template <int KL>
__device__ __forceinline__ void knn_pk_consider(float* key, float* rej, int j, unsigned code, V2 p, float r2,
                                                const V2* s_pos)
{
    const V2 q = s_pos[j];
    const float dx = q.x - p.x, dy = q.y - p.y;
    const float d2 = dx * dx + dy * dy; /* KDTree.cpp:107-108 */
    if (!(d2 > kEps) || !(d2 < r2)) return;
    float nk = __uint_as_float((__float_as_uint(d2) & ~kCodeMask) | code);
    if (nk < key[KL - 1]) {
        /* every entry from the old list alone (no chain through the list):
           entry q becomes min(old q, max(old q-1, nk)); the entry pushed out
           is max(old last, nk) */
        const float out = fmaxf(key[KL - 1], nk);
#pragma unroll
        for (int q2 = KL - 1; q2 > 0; q2--) key[q2] = fminf(key[q2], fmaxf(key[q2 - 1], nk));
        key[0] = fminf(key[0], nk);
        nk = out;
    }
    *rej = fminf(*rej, nk);
}

/* grid index of a packed key's candidate */
__device__ __forceinline__ int knn_pk_index(float k, int cx, int cy, int sx, int sy, const int* cell_start,
                                            const AgentGrid& g)
{
    const unsigned code = __float_as_uint(k) & kCodeMask;
    const int i = (int)(code >> 5), off = (int)(code & 31u);
    if (i == kCodeOverflow) return cell_start[g.ncells] + off;
    const int x = cx + sx * (int)c_knn_tmpl.dx[i], y = cy + sy * (int)c_knn_tmpl.dy[i];
    return cell_start[y * g.gw + x] + off;
}

/* where a packed list's codes point: the agent's cell and mirror signs */
struct PkFrame {
    int cx, cy, sx, sy;
};

/* the packed list of KL entries */
template <int KL>
struct PkList {
    float key[KL];
};

/* near ties in the list (rare; out of line): the valid entries from lo on
   decoded, re-sorted by the exact (d2, slot) key and the first k written to
   o[0 .. k) (-1 beyond the count) */
template <int KL>
__device__ __noinline__ void knn_pk_write_exact(PkList<KL> L, int lo, int k, PkFrame f, V2 p, const V2* s_pos,
                                                const int* s_slot, const int* cell_start, AgentGrid g, int* o)
{
    unsigned long long ek[KL];
    int id[KL];
    int n = 0;
    for (int q = lo; q < KL; q++) {
        if (!(L.key[q] < INFINITY)) break;
        const int j = knn_pk_index(L.key[q], f.cx, f.cy, f.sx, f.sy, cell_start, g);
        const V2 c = s_pos[j];
        const float dx = c.x - p.x, dy = c.y - p.y;
        const float d2 = dx * dx + dy * dy;
        ek[n] = ((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)s_slot[j];
        id[n] = j;
        n++;
    }
    for (int q = 1; q < n; q++) {
        for (int r = q; r > 0 && ek[r - 1] > ek[r]; r--) {
            const unsigned long long t = ek[r];
            ek[r] = ek[r - 1];
            ek[r - 1] = t;
            const int ti = id[r];
            id[r] = id[r - 1];
            id[r - 1] = ti;
        }
    }
    for (int q = 0; q < k; q++) o[q] = q < n ? id[q] : -1;
}

/* 1: the packed list in *L is exact apart from near ties inside it (2: with
   such ties); 0: the caller must run the 64-bit search.  *cnt = count. */
template <int K>
__device__ __forceinline__ int knn_fast(PkList<K + 2>* L, PkFrame* f, int k, V2 p, float r2, const V2* s_pos,
                                        const int* cell_start, const AgentGrid& g, int* cnt)
{
    constexpr int KL = K + 2; /* two entries beyond the k-th */
    float* key = L->key;
#pragma unroll
    for (int q = 0; q < KL; q++) key[q] = q < K - k ? 0.0f : INFINITY; /* 0: below every candidate */
    float rej = INFINITY;
    const int o0 = cell_start[g.ncells], o1 = cell_start[g.ncells + 1];
    if (o1 - o0 > 32) return 0;
    for (int j = o0; j < o1; j++)
        knn_pk_consider<KL>(key, &rej, j, (unsigned)(kCodeOverflow << 5) | (unsigned)(j - o0), p, r2, s_pos);
    const float fx = (p.x - g.x0) * g.inv, fy = (p.y - g.y0) * g.inv;
    if (!(fx >= 0.0f && fy >= 0.0f && fx < (float)g.gw && fy < (float)g.gh)) return 0;
    const int cx = (int)fx, cy = (int)fy;
    const int sx = fx - (float)cx < 0.5f ? 1 : -1, sy = fy - (float)cy < 0.5f ? 1 : -1;
    f->cx = cx;
    f->cy = cy;
    f->sx = sx;
    f->sy = sy;
    const float half = 0.5f * g.cell;
    bool crowded = false;
    int i = 0;
    for (; i < kTmplN; i++) {
        /* the largest d2 the k-th entry can stand for */
        const float kd = fminf(r2, __uint_as_float(__float_as_uint(key[K - 1]) | kCodeMask));
        /* every later cell is at least this far from the agent (1 cm for the
           rounding of the bucket assignment) */
        const float bx = fmaxf((float)c_knn_tmpl.hx[i] * half - 0.01f, 0.0f);
        const float by = fmaxf((float)c_knn_tmpl.hy[i] * half - 0.01f, 0.0f);
        if (bx * bx + by * by > kd) break;
        const int x = cx + sx * (int)c_knn_tmpl.dx[i], y = cy + sy * (int)c_knn_tmpl.dy[i];
        if (x < 0 || y < 0 || x >= g.gw || y >= g.gh) continue;
        const float rx0 = g.x0 + (float)x * g.cell, ry0 = g.y0 + (float)y * g.cell;
        const float ex = fmaxf(fmaxf(rx0 - p.x, p.x - (rx0 + g.cell)) - 0.01f, 0.0f);
        const float ey = fmaxf(fmaxf(ry0 - p.y, p.y - (ry0 + g.cell)) - 0.01f, 0.0f);
        if (ex * ex + ey * ey > kd) continue;
        const int c = y * g.gw + x;
        const int j0 = cell_start[c], j1 = cell_start[c + 1];
        crowded |= j1 - j0 > 32;
        const unsigned base = (unsigned)i << 5;
        for (int j = j0; j < j1; j++) knn_pk_consider<KL>(key, &rej, j, base | (unsigned)(j - j0), p, r2, s_pos);
    }
    if (i == kTmplN || crowded) return 0;
    int n = 0;
    bool tie = false;
#pragma unroll
    for (int q = 0; q < KL; q++) {
        if (q < K - k || !(key[q] < INFINITY)) continue;
        if (q < K) n++;
        if (q + 1 < KL && key[q + 1] < INFINITY && key_hi(key[q + 1]) == key_hi(key[q])) tie = true;
    }
    /* a dropped candidate may share the k-th entry's leading bits only when
       the group reaches the list's last entry */
    if (n == k && key[KL - 1] < INFINITY && key_hi(key[KL - 1]) == key_hi(key[K - 1]) &&
        key_hi(rej) == key_hi(key[K - 1]))
        return 0;
    *cnt = n;
    return tie ? 2 : 1;
}

/* ---------------------------------------------------------------------- */
struct LocalGet {
    const Con* c;
    __device__ Con operator()(int i) const { return c[i]; }
};

/* adds the number of lanes with pred set to *ctr with one atomic per warp */
__device__ __forceinline__ void warp_count(int* ctr, bool pred)
{
    unsigned m = __activemask();
    unsigned b = __ballot_sync(m, pred);
    if ((threadIdx.x & 31) == __ffs(m) - 1 && b) atomicAdd(ctr, __popc(b));
}

/* class of an LP result for the proposal's training labels (kCls*) */
__device__ __forceinline__ int label_of(const LpTrace& tr, int failed, int m, int nObst)
{
    if (failed < m) return kClsOther;
    if (tr.h < 0) return kClsPref;
    int q = tr.h - nObst;
    if (q < 0 || q >= kMlpNbrs) return kClsOther;
    if (tr.src == 0) return kClsSingle + q;
    if (tr.src == 1) return kClsCircle + q;
    int qj = tr.j - nObst;
    if (qj < 0) return kClsOther;
    return kClsPair + q * (q - 1) / 2 + qj;
}

/* Exact check of a proposed active set.  Returns true only when the
   incremental LP (lp2d, ORCA.cpp:428-587) provably ends with its last update
   on the proposed half-plane h, fixed by the proposed bound; *out is then
   computed with the LP's own final-step formula, so it is the LP's result.
   Conditions: the bounds of h over every earlier half-plane and the speed
   circle reproduce the proposed source; every later half-plane contains the
   point (the LP's own test); the KKT multipliers of the proposed active set
   are positive and every other earlier half-plane is slack, both by a margin,
   so that the LP state before h violates h. */
template <class Get>
__device__ __noinline__ bool verify_proposal(const Get& get, int m, int nObst, int ncnt, V2 opt, float maxSpeed,
                                             int cls, V2* out)
{
    const float margin = 1e-4f;
    if (cls == kClsPref) {
        V2 v0 = (len(opt) > maxSpeed) ? normalized(opt) * maxSpeed : opt;
        for (int i = 0; i < m; i++) {
            Con c = get(i);
            if (det(right(c.n), c.p - v0) > 0.0f) return false;
        }
        *out = v0;
        return true;
    }
    int q, qj = -1, kind; /* kind 0 single, 1 circle, 2 pair */
    if (cls >= kClsSingle && cls < kClsPair) { q = cls - kClsSingle; kind = 0; }
    else if (cls >= kClsCircle && cls < kClsOther) { q = cls - kClsCircle; kind = 1; }
    else if (cls >= kClsPair && cls < kClsCircle) {
        int p = cls - kClsPair;
        q = 1;
        while ((q + 1) * q / 2 <= p) q++; /* q*(q-1)/2 <= p < (q+1)*q/2 */
        qj = p - q * (q - 1) / 2;
        kind = 2;
    } else return false;
    if (q >= ncnt || q >= kMlpNbrs) return false;
    const int h = nObst + q, jsrc = kind == 2 ? nObst + qj : -1;
    if (h >= m) return false;
    Con H = get(h);
    V2 dir = right(H.n);
    float dpd = dot(dir, H.p);
    float disc = dpd * dpd + maxSpeed * maxSpeed - dot(H.p, H.p);
    if (!(disc > 0.0f)) return false;
    float sq = sqrtf(disc);
    float lo = -dpd - sq, hi = -dpd + sq;
    int lo_src = -1, hi_src = -1;
    for (int j = 0; j < h; j++) {
        Con G = get(j);
        float den = det(right(H.n), right(G.n));
        float num = det(right(G.n), H.p - G.p);
        if (fabsf(den) <= kEps) {
            if (num < 0.0f) return false;
            continue;
        }
        const float t = num / den;
        if (den >= 0.0f) {
            if (t < hi) hi_src = j;
            hi = (t < hi) ? t : hi;
        } else {
            if (lo < t) lo_src = j;
            lo = (lo < t) ? t : lo;
        }
    }
    if (lo > hi) return false;
    float t = dot(dir, opt - H.p);
    V2 v;
    int src; /* -2 projection, -1 circle, else constraint index */
    if (t < lo) { v = H.p + dir * lo; src = lo_src; }
    else if (t > hi) { v = H.p + dir * hi; src = hi_src; }
    else { v = H.p + dir * t; src = -2; }
    if (kind == 0 && src != -2) return false;
    if (kind == 1 && src != -1) return false;
    if (kind == 2 && src != jsrc) return false;
    for (int i = h + 1; i < m; i++) {
        Con c = get(i);
        if (det(right(c.n), c.p - v) > 0.0f) return false;
    }
    /* KKT of min |v - opt|^2 s.t. dot(N_i, v - P_i) >= 0, |v| <= maxSpeed */
    V2 r = v - opt;
    if (kind != 1) { /* the speed circle must be slack as well */
        float rs = maxSpeed - margin;
        if (!(rs > 0.0f && dot(v, v) < rs * rs)) return false;
    }
    if (kind == 0) {
        if (!(dot(r, H.n) > margin)) return false;
    } else if (kind == 2) {
        Con G = get(jsrc);
        float d2 = det(H.n, G.n);
        float la = det(r, G.n) / d2, lb = det(H.n, r) / d2;
        if (!(la > margin && lb > margin)) return false;
    } else {
        V2 nv = v * -1.0f;
        float d2 = det(H.n, nv);
        if (!(fabsf(d2) > kEps)) return false;
        float la = det(r, nv) / d2, lb = det(H.n, r) / d2;
        if (!(la > margin && lb > margin * maxSpeed)) return false;
    }
    for (int i = 0; i < h; i++) {
        if (i == jsrc) continue;
        Con c = get(i);
        if (!(det(right(c.n), c.p - v) < -margin)) return false;
    }
    *out = v;
    return true;
}

/* out-of-line copies keep the per-agent kernel small enough for the
   instruction cache: each is called from a loop or a rare branch */
__device__ __noinline__ Con agent_constraint_ni(V2 position, V2 velocity, float clr, V2 np, V2 nv, float nclr,
                                                float tau, float dt, float inv_tau)
{
    return agent_constraint(position, velocity, clr, np, nv, nclr, tau, dt, inv_tau);
}

template <int MC>
__device__ __noinline__ void lp3d_local(const Con* cons, int m, int nObst, float maxSpeed, int failed, V2* v,
                                        bool fp64)
{
    Con proj[MC - kMaxObstCons]; /* bisectors: at most the neighbour constraints */
    LocalGet get{cons};
    lp3d(get, m, nObst, maxSpeed, failed, v, proj, fp64);
}

/* attraction point and preferred velocity of grid-order agent t */
__device__ void attract_tick(const TickArgs& a, int t)
{
    const int slot = a.s_slot[t];
    if (a.active[slot] & kActivePending) return; /* done by k_fixup once its new path is in */
    const V2 pos = a.s_pos[t];
    const SceneDev& sc = a.scenes[a.slot_scene ? a.slot_scene[slot] : 0];
    /* the point location of the retraction, issued before the path loads
       (independent chains of dependent loads); unused when the agent arrives */
    const int cell = point_location_inl(sc.ecm, pos);

    /* UpdateAttractionPointSystem (Simulator.cpp:538-590) */
    const int off = a.path_off[slot], np = a.path_len[slot];
    const V2* path = a.path_xy + off;
    const V2 goal = path[np - 1];
    float gdx = pos.x - goal.x, gdy = pos.y - goal.y;
    float dist = gdx * gdx + gdy * gdy;
    V2 attr;
    if (dist < a.arr_sq) {
        attr = goal;
        a.attr[slot] = attr;
        if (dist < a.del_sq) { /* DestroyAgent: skipped by every later system */
            a.active[slot] = 0;
            int q = atomicAdd(&a.counters[C_DESTROYED], 1);
            if (q < a.list_cap) a.destroyed_list[q] = slot;
            else atomicOr(&a.counters[C_ERROR], ECMG_DEV_ERR_LIST);
            if (a.rec_cnt) a.rec_cnt[slot] = -1;
            return;
        }
    } else {
        V2 ap = mk(0.0f, 0.0f); /* Point attractionPoint; (0,0) */
        bool no_retract = false;
        int red = -1;
        if (irm(sc.ecm, pos, path, np, &ap, &no_retract, &red, cell)) {
            attr = ap;
            a.attr[slot] = attr;
        } else if (a.replan_dev_fail && (no_retract || (red >= 0 && a.fail_edge[slot] == red))) {
            /* the built-in planner starts by retracting this same position
               with the same point location; it fails there, or its search
               already failed from this ECM edge for this goal and clearance
               (a property of the edge only).  Either way the re-plan fails:
               the agent keeps its path and attraction point without a host
               round trip. */
            attr = a.attr[slot];
            atomicAdd(&a.counters[C_REPLAN_DEV], 1);
        } else {
            attr = a.attr[slot]; /* unchanged; the host re-plans before the next tick */
            int q = atomicAdd(&a.counters[C_REPLAN], 1);
            if (q < a.list_cap) { a.replan_list[q] = slot; a.replan_pos[q] = pos; }
            else atomicOr(&a.counters[C_ERROR], ECMG_DEV_ERR_LIST);
        }
    }

    /* ApplySteeringForce (Simulator.cpp:638-657) */
    const float speed = a.speed[slot];
    V2 pv = normalize(attr - pos) * speed;
    a.pref_vel[slot] = pv;
}

/* ApplyObstacleAvoidanceForce + UpdateVelocitySystem + UpdatePositionSystem
   of grid-order agent t (agents destroyed this tick are skipped).  FULL
   keeps the learned proposal's check, the trace labels and the recording of
   the step; the plain tick's kernel is compiled without them (smaller code,
   the same arithmetic). */
template <int K, bool FULL = true>
__device__ void orca_tick(const TickArgs& a, int t)
{
    const int slot = a.s_slot[t];
    if (a.active[slot] != 1) return; /* inactive, or waiting for its re-plan (k_fixup) */
    const V2 pos = a.s_pos[t];
    const V2 vel = a.s_vel[t];
    const float clr = a.s_clear[t];
    const SceneDev& sc = a.scenes[a.slot_scene ? a.slot_scene[slot] : 0];
    const float speed = a.speed[slot];
    const V2 pv = a.pref_vel[slot];

    /* ORCA::GetVelocity (ORCA.cpp:14-57) with maxSpeed = preferred speed
       (Simulator.cpp:671) unless a global maximum is configured */
    const float maxSpeed = a.max_speed > 0.0f ? a.max_speed : speed;
    const int ncnt = a.ncnt[t];
    const int* nbr = a.nbr + (size_t)t * a.k;
    constexpr int MC = K + kMaxObstCons; /* constraint capacity */
    Con cons[MC];
    LocalGet get{cons};
    /* the plain tick takes each constraint into RandomizedLP as soon as it is
       built (the LP's steps in the same order as over the finished list) */
    V2 v = lp2d_start(pv, maxSpeed, false);
    int failed2 = -1;
    int m = 0;
    bool overflow = false;
    const float range = a.tau_o * maxSpeed + clr;
    const float rsq = range * range;
    {
        const ObstView& o = sc.ob;
        int b = 0, e = 0;
        const int* items = nullptr;
        float fx = (pos.x - o.gx0) * o.ginv, fy = (pos.y - o.gy0) * o.ginv;
        if (o.g_start && range <= o.reach && fx >= 0.0f && fy >= 0.0f && fx < (float)o.gw && fy < (float)o.gh) {
            int g = (int)fy * o.gw + (int)fx;
            b = o.g_start[g];
            e = o.g_start[g + 1];
            items = o.g_items;
        } else {
            e = o.n_verts; /* linear scan: the reference's own loop */
        }
        for (int q = b; q < e; q++) {
            int L = items ? items[q] : q;
            if (!obstacle_in_range(o, L, pos, rsq)) continue;
            Con c;
            if (obstacle_constraint_inl(o, L, pos, vel, clr, a.tau_o, &c)) {
                if (m < MC - K) {
                    cons[m] = c;
                    if (!FULL && failed2 < 0 && !lp2d_step(get, m, c, pv, maxSpeed, false, &v)) failed2 = m;
                    m++;
                } else {
                    overflow = true;
                }
            }
        }
    }
    const int nObst = m;
    for (int q = 0; q < ncnt; q++) {
        const int j = nbr[q];
        if (j >= 0) {
            /* inline in the plain kernel (no other callers compete for the
               instruction cache there), out of line in the full one */
            cons[m] = agent_constraint(pos, vel, clr, a.s_pos[j], a.s_vel[j], a.s_clear[j], a.tau_a, a.dt,
                                       a.inv_tau_a);
        } else {
            /* kd-tree mode: a cache entry left by an earlier agent that is
               not in this tick's grid; its slot is not written this tick */
            const int sl = -j - 1;
            cons[m] = agent_constraint_ni(pos, vel, clr, a.pos[sl], a.vel[sl], a.clear[sl], a.tau_a, a.dt,
                                          a.inv_tau_a);
        }
        if (!FULL && failed2 < 0 && !lp2d_step(get, m, cons[m], pv, maxSpeed, false, &v)) failed2 = m;
        m++;
    }
    if (overflow) atomicOr(&a.counters[C_ERROR], ECMG_DEV_ERR_CONSTRAINTS);

    int failed = -1;
    if (FULL && (a.cls || a.cls_slot)) { /* learned proposal: accepted only when the exact check passes */
        const int c = a.cls_slot ? a.cls_slot[slot] : a.cls[t];
        bool ok = c != kClsOther && verify_proposal(get, m, nObst, ncnt, pv, maxSpeed, c, &v);
        if (ok) failed = m;
        warp_count(&a.counters[C_PROPOSED], c != kClsOther);
        warp_count(&a.counters[C_ACCEPTED], ok);
    }
    bool need3d = false;
    if (failed < 0) {
        if (FULL && a.label) {
            LpTrace tr;
            failed = lp2d<LocalGet, true>(get, m, pv, maxSpeed, false, &v, &tr);
            a.label[t] = (unsigned char)label_of(tr, failed, m, nObst);
        } else if (FULL) {
            failed = lp2d(get, m, pv, maxSpeed, false, &v);
        } else {
            failed = failed2 < 0 ? m : failed2;
        }
        if (failed < m) {
            lp3d_local<MC>(cons, m, nObst, maxSpeed, failed, &v, a.lp3d_fp64 != 0);
            need3d = true;
        }
    }
    warp_count(&a.counters[C_LP3D], need3d);

    /* force = vOrca - v (Simulator.cpp:676-677); UpdateVelocitySystem
       (Simulator.cpp:619-635); UpdatePositionSystem (Simulator.cpp:592-606) */
    float fx = v.x - vel.x, fy = v.y - vel.y;
    V2 nv = mk(vel.x + fx * a.mass_recip * a.dt, vel.y + fy * a.mass_recip * a.dt);
    V2 npos = mk(pos.x + (nv.x * a.dt), pos.y + (nv.y * a.dt));
    a.vel[slot] = nv;
    a.pos[slot] = npos;

    if (FULL && a.rec_cnt) {
        a.rec_cnt[slot] = ncnt;
        for (int q = 0; q < a.k; q++)
            a.rec_nbr[slot * a.k + q] = q < ncnt ? (nbr[q] >= 0 ? a.s_slot[nbr[q]] : -nbr[q] - 1) : -1;
        a.rec_vorca[slot] = v;
        a.rec_fail[slot] = failed;
        a.rec_ncons[slot] = m;
        a.rec_nobst[slot] = nObst;
    }
}

/* the 64-bit (d2, slot) search of grid-order agent t (rare: equal
   distances, sparse crowds, agents outside the grid); out of line so that it
   does not take registers from the fast path */
template <int K>
__device__ __noinline__ void knn_agent_exact(const TickArgs& a, int t, const SceneDev& sc)
{
    Knn<K> nn;
    knn_grid<K>(nn, a.k, a.s_pos[t], a.rnb, a.rnb2, a.s_pos, a.s_slot, a.cell_start + sc.bucket_base, sc.grid);
    a.ncnt[t] = nn.cnt;
    int* o = a.nbr + (size_t)t * a.k;
#pragma unroll
    for (int q2 = 0; q2 < K; q2++) {
        const int q = q2 - (K - a.k);
        if (q >= 0) {
            const int sl = (int)(unsigned)nn.key[q2];
            o[q] = q < nn.cnt ? a.cell_start[a.slot_bucket[sl]] + a.slot_rank[sl] : -1;
        }
    }
}

/* neighbour lists of every grid-order agent of the tick (KNearestAgents,
   KDTree.cpp:85-202, as the exact (d2, slot) query of the grid) */
template <int K>
__device__ __forceinline__ void knn_agent(const TickArgs& a, int t, int slot)
{
    const SceneDev& sc = a.scenes[a.slot_scene ? a.slot_scene[slot] : 0];
    const int* cs = a.cell_start + sc.bucket_base;
    const V2 p = a.s_pos[t];
    PkList<K + 2> L;
    PkFrame f;
    int n = 0;
    const int st = knn_fast<K>(&L, &f, a.k, p, a.rnb2, a.s_pos, cs, sc.grid, &n);
    if (st != 0) {
        a.ncnt[t] = n;
        int* o = a.nbr + (size_t)t * a.k;
        if (st == 1) {
#pragma unroll
            for (int q2 = 0; q2 < K; q2++) {
                const int q = q2 - (K - a.k);
                if (q >= 0) o[q] = q < n ? knn_pk_index(L.key[q2], f.cx, f.cy, f.sx, f.sy, cs, sc.grid) : -1;
            }
        } else {
            knn_pk_write_exact<K + 2>(L, K - a.k, a.k, f, p, a.s_pos, a.s_slot, cs, sc.grid, o);
        }
        return;
    }
    knn_agent_exact<K>(a, t, sc);
}

/* persistent: a warp takes 32 consecutive grid-order agents per work grab
   (neighbouring agents: their candidates share L1), so that warps whose
   agents have more candidates do not leave the SMs' last wave ragged */
template <int K, int MINB>
__global__ void __launch_bounds__(128, MINB) k_neighbors(TickArgs a)
{
    const int n = a.counters[C_NSORTED];
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&a.counters[C_NBR_WORK], 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int t = base + lane;
        if (t < n) knn_agent<K>(a, t, a.s_slot[t]);
    }
}

/* UpdateAttractionPointSystem + ApplySteeringForce for every agent */
__global__ void __launch_bounds__(128) k_attract(TickArgs a)
{
    const int n = a.counters[C_NSORTED];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) attract_tick(a, t);
}

/* agents whose re-plan is still being computed on the host when the tick
   starts: the tick's attraction and ORCA kernels skip them */
__global__ void k_mark_pending(TickArgs a, const int* list, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        a.active[list[i]] |= kActivePending;
}

/* the skipped step of those agents, after the tick's kernels and the upload
   of their new paths: UpdateAttractionPointSystem with the new path, then
   ApplyObstacleAvoidanceForce and the integration on the tick's snapshot and
   neighbour lists (still in place until the next tick's binning) -- the
   same functions on the same inputs as the tick's own kernels */
template <int K, bool FULL>
__global__ void __launch_bounds__(128) k_fixup(TickArgs a, const int* list, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int slot = list[i];
        if (!(a.active[slot] & kActivePending)) continue;
        a.active[slot] = 1;
        const int t = a.cell_start[a.slot_bucket[slot]] + a.slot_rank[slot];
        attract_tick(a, t);
        orca_tick<K, FULL>(a, t);
    }
}

/* proposal features of every grid-order agent (zeros for agents destroyed
   this tick): 16 neighbours x (relative position / neighbour distance,
   relative velocity / 2, radius sum), preferred velocity / LP radius */
__global__ void __launch_bounds__(128) k_features(TickArgs a)
{
    const int n = a.counters[C_NSORTED];
    __nv_bfloat16* F = (__nv_bfloat16*)a.feat;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        float f[kMlpIn];
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
        const int slot = a.s_slot[t];
        if (a.active[slot]) {
            const V2 pos = a.s_pos[t], vel = a.s_vel[t];
            const float clr = a.s_clear[t];
            const float speed = a.speed[slot];
            const float maxSpeed = a.max_speed > 0.0f ? a.max_speed : speed;
            const int ncnt = a.ncnt[t];
            const int* nbr = a.nbr + (size_t)t * a.k;
            const float inv_r = 1.0f / a.rnb;
#pragma unroll
            for (int q = 0; q < kMlpNbrs; q++) {
                if (q < ncnt) {
                    int j = nbr[q];
                    V2 pj = a.s_pos[j], vj = a.s_vel[j];
                    f[5 * q + 0] = (pj.x - pos.x) * inv_r;
                    f[5 * q + 1] = (pj.y - pos.y) * inv_r;
                    f[5 * q + 2] = (vel.x - vj.x) * 0.5f;
                    f[5 * q + 3] = (vel.y - vj.y) * 0.5f;
                    f[5 * q + 4] = a.s_clear[j] + clr;
                }
            }
            V2 pv = a.pref_vel[slot];
            float im = maxSpeed > 0.0f ? 1.0f / maxSpeed : 0.0f;
            f[5 * kMlpNbrs] = pv.x * im;
            f[5 * kMlpNbrs + 1] = pv.y * im;
        }
        uint4* row = reinterpret_cast<uint4*>(F + (size_t)t * kMlpIn);
#pragma unroll
        for (int c = 0; c < kMlpIn / 8; c++) {
            __nv_bfloat162 h0 = __floats2bfloat162_rn(f[8 * c + 0], f[8 * c + 1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(f[8 * c + 2], f[8 * c + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(f[8 * c + 4], f[8 * c + 5]);
            __nv_bfloat162 h3 = __floats2bfloat162_rn(f[8 * c + 6], f[8 * c + 7]);
            uint4 u;
            u.x = *reinterpret_cast<unsigned*>(&h0);
            u.y = *reinterpret_cast<unsigned*>(&h1);
            u.z = *reinterpret_cast<unsigned*>(&h2);
            u.w = *reinterpret_cast<unsigned*>(&h3);
            row[c] = u;
        }
    }
}

/* persistent kernel: a warp takes `tile` consecutive grid-order agents per
   work grab (one atomic per grab) and runs them 32 at a time */
template <int K, bool FULL>
__global__ void __launch_bounds__(256, (K <= 16) ? 4 : 1) k_agents(TickArgs a)
{
    const int n = a.counters[C_NSORTED];
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&a.counters[C_WORK], a.tile);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        for (int o = 0; o < a.tile; o += 32) {
            int t = base + o + lane;
            if (t < n) orca_tick<K, FULL>(a, t);
        }
    }
}

/* the per-thread layout fused with the neighbour search (ECMG_LP_THREAD_FUSED):
   each thread finds its agent's k nearest, then runs the agent's step, so
   that warps in the ALU-bound search and warps in the issue-bound LPs share
   every SM.  Agents destroyed by the attraction kernel get no list (no later
   stage of a plain tick reads it). */
template <int K, bool FULL>
__global__ void __launch_bounds__(256) k_agents_knn(TickArgs a)
{
    const int n = a.counters[C_NSORTED];
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&a.counters[C_WORK], a.tile);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        for (int o = 0; o < a.tile; o += 32) {
            const int t = base + o + lane;
            if (t >= n) continue;
            const int slot = a.s_slot[t];
            if (!a.active[slot]) continue;
            knn_agent<K>(a, t, slot);
            orca_tick<K, FULL>(a, t);
        }
    }
}

/* ------------------------------------------------------------------------
 * Warp-cooperative per-agent step: one warp per agent.  The lanes build the
 * obstacle and neighbour constraints in parallel and keep them in shared
 * memory in the reference's order (ballot compaction preserves the candidate
 * order).  The incremental LPs stay sequential over the constraint index i;
 * the bounds of line i from the lines j < i are spread over the lanes and
 * combined by min/max reductions that keep the first j on ties.  min/max are
 * exact, the per-element arithmetic is the per-thread code's, and "some line
 * is parallel and opposite" / "lo > hi" are order-free predicates, so the
 * results equal the per-thread LP's bit for bit.
 * ---------------------------------------------------------------------- */
constexpr unsigned kFull = 0xffffffffu;

struct SmemGet {
    const Con* c;
    __device__ Con operator()(int i) const { return c[i]; }
};

/* projected lines of RandomizedLP3D: the obstacle constraints, then the
   bisectors */
struct ProjGetW {
    const Con* obs;
    const Con* bis;
    int nObst;
    __device__ Con operator()(int i) const { return i < nObst ? obs[i] : bis[i - nObst]; }
};

/* lo/hi bounds on line h from the lines j < i (ORCA.cpp:461-497), lanes
   taking j = lane, lane + 32, ...; false when a parallel line excludes h */
template <class Get>
__device__ __forceinline__ bool warp_bounds(const Get& get, const Con& h, int i, int lane, float* lo, float* hi,
                                            int* lo_src, int* hi_src)
{
    float llo = -INFINITY, lhi = INFINITY;
    int jlo = 0x7fffffff, jhi = 0x7fffffff;
    bool bad = false;
    const V2 rh = right(h.n);
    for (int j = lane; j < i; j += 32) {
        Con g = get(j);
        float den = det(rh, right(g.n));
        float num = det(right(g.n), h.p - g.p);
        if (fabsf(den) <= kEps) {
            if (num < 0.0f) bad = true;
            continue;
        }
        const float t = num / den;
        if (den >= 0.0f) {
            if (t < lhi) { lhi = t; jhi = j; }
        } else {
            if (llo < t) { llo = t; jlo = j; }
        }
    }
    if (__any_sync(kFull, bad)) return false;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        float v = __shfl_xor_sync(kFull, lhi, o);
        int jj = __shfl_xor_sync(kFull, jhi, o);
        if (v < lhi || (v == lhi && jj < jhi)) { lhi = v; jhi = jj; }
        v = __shfl_xor_sync(kFull, llo, o);
        jj = __shfl_xor_sync(kFull, jlo, o);
        if (llo < v || (v == llo && jj < jlo)) { llo = v; jlo = jj; }
    }
    if (lhi < *hi) { *hi = lhi; *hi_src = jhi; }
    if (*lo < llo) { *lo = llo; *lo_src = jlo; }
    return true;
}

/* RandomizedLP (ORCA.cpp:428-587) for a whole warp; every lane returns the
   same result */
template <class Get, bool TRACE>
__device__ int lp2d_warp(const Get& get, int n, V2 opt, float maxSpeed, bool useDirOpt, V2* out, LpTrace* tr,
                         int lane)
{
    V2 v;
    if (useDirOpt) v = opt * maxSpeed;
    else if (len(opt) > maxSpeed) v = normalized(opt) * maxSpeed;
    else v = opt;
    for (int i = 0; i < n; i++) {
        const Con h = get(i);
        if (det(right(h.n), h.p - v) <= 0.0f) continue; /* Constraint::Contains */
        const V2 dir = right(h.n);
        const float dpd = dot(dir, h.p);
        const float disc = dpd * dpd + maxSpeed * maxSpeed - dot(h.p, h.p);
        if (disc <= 0.0f) { *out = v; return i; }
        if (!(disc > 0.0f)) continue; /* NaN: passed over (ORCA.cpp:498-506) */
        const float sq = sqrtf(disc);
        float lo = -dpd - sq, hi = -dpd + sq;
        int lo_src = -1, hi_src = -1;
        if (!warp_bounds(get, h, i, lane, &lo, &hi, &lo_src, &hi_src) || lo > hi) { *out = v; return i; }
        if (useDirOpt) {
            if (dot(opt, dir) > 0) v = h.p + dir * hi;
            else v = h.p + dir * lo;
        } else {
            const float t = dot(dir, opt - h.p);
            if (t < lo) {
                v = h.p + dir * lo;
                if (TRACE) { tr->h = i; tr->src = lo_src < 0 ? 1 : 2; tr->j = lo_src; }
            } else if (t > hi) {
                v = h.p + dir * hi;
                if (TRACE) { tr->h = i; tr->src = hi_src < 0 ? 1 : 2; tr->j = hi_src; }
            } else {
                v = h.p + dir * t;
                if (TRACE) { tr->h = i; tr->src = 0; tr->j = -1; }
            }
        }
    }
    *out = v;
    return n;
}

/* RandomizedLP3D (ORCA.cpp:592-669) for a whole warp: the bisectors of
   line i are built by the lanes (compacted in j order), the projected LP is
   lp2d_warp.  bis holds at least m - nObst lines. */
__device__ __noinline__ void lp3d_warp(const Con* cons, Con* bis, int m, int nObst, float maxSpeed, int failed,
                                       V2* vout, bool fp64, int lane)
{
    V2 v = *vout;
    float maxPen = 0.0f;
    for (int i = failed; i < m; i++) {
        const Con ci = cons[i];
        const V2 dir = right(ci.n);
        if (det(dir, ci.p - v) <= maxPen) continue;
        int cnt = 0;
        for (int base = nObst; base < i; base += 32) {
            const int j = base + lane;
            bool keep = false;
            Con nc;
            if (j < i) {
                const Con cj = cons[j];
                const float dt = det(right(ci.n), right(cj.n));
                if (fabsf(dt) <= kEps) {
                    if (!(dot(ci.n, cj.n) > 0)) {
                        nc.p = (ci.p + cj.p) * 0.5f;
                        keep = true;
                    }
                } else if (!fp64) {
                    const float t = det(right(cj.n), ci.p - cj.p) / dt;
                    nc.p = ci.p + right(ci.n) * t;
                    keep = true;
                } else {
                    double ax = (double)cj.n.y, ay = -(double)cj.n.x;
                    double bx = (double)ci.p.x - (double)cj.p.x, by = (double)ci.p.y - (double)cj.p.y;
                    double rx = (double)ci.n.y, ry = -(double)ci.n.x;
                    double dd = rx * ay - ry * ax;
                    double t = (ax * by - ay * bx) / dd;
                    nc.p = mk((float)((double)ci.p.x + rx * t), (float)((double)ci.p.y + ry * t));
                    keep = true;
                }
                if (keep) nc.n = normalized(cj.n - ci.n);
            }
            const unsigned b = __ballot_sync(kFull, keep);
            if (keep) bis[cnt + __popc(b & ((1u << lane) - 1u))] = nc;
            cnt += __popc(b);
        }
        __syncwarp();
        const V2 temp = v;
        ProjGetW pg{cons, bis, nObst};
        if (lp2d_warp<ProjGetW, false>(pg, nObst + cnt, ci.n, maxSpeed, true, &v, nullptr, lane) < nObst + cnt)
            v = temp;
        maxPen = det(dir, ci.p - v);
        __syncwarp(); /* bis is rewritten for the next line */
    }
    *vout = v;
}

/* verify_proposal for a whole warp (same conditions, lanes over the
   constraints) */
__device__ __noinline__ bool verify_proposal_warp(const Con* cons, int m, int nObst, int ncnt, V2 opt, float maxSpeed,
                                                  int cls, V2* out, int lane)
{
    const float margin = 1e-4f;
    SmemGet get{cons};
    if (cls == kClsPref) {
        V2 v0 = (len(opt) > maxSpeed) ? normalized(opt) * maxSpeed : opt;
        bool bad = false;
        for (int i = lane; i < m; i += 32) {
            Con c = cons[i];
            if (det(right(c.n), c.p - v0) > 0.0f) bad = true;
        }
        if (__any_sync(kFull, bad)) return false;
        *out = v0;
        return true;
    }
    int q, qj = -1, kind;
    if (cls >= kClsSingle && cls < kClsPair) { q = cls - kClsSingle; kind = 0; }
    else if (cls >= kClsCircle && cls < kClsOther) { q = cls - kClsCircle; kind = 1; }
    else if (cls >= kClsPair && cls < kClsCircle) {
        int p = cls - kClsPair;
        q = 1;
        while ((q + 1) * q / 2 <= p) q++;
        qj = p - q * (q - 1) / 2;
        kind = 2;
    } else return false;
    if (q >= ncnt || q >= kMlpNbrs) return false;
    const int h = nObst + q, jsrc = kind == 2 ? nObst + qj : -1;
    if (h >= m) return false;
    const Con H = cons[h];
    const V2 dir = right(H.n);
    const float dpd = dot(dir, H.p);
    const float disc = dpd * dpd + maxSpeed * maxSpeed - dot(H.p, H.p);
    if (!(disc > 0.0f)) return false;
    const float sq = sqrtf(disc);
    float lo = -dpd - sq, hi = -dpd + sq;
    int lo_src = -1, hi_src = -1;
    if (!warp_bounds(get, H, h, lane, &lo, &hi, &lo_src, &hi_src) || lo > hi) return false;
    const float t = dot(dir, opt - H.p);
    V2 v;
    int src;
    if (t < lo) { v = H.p + dir * lo; src = lo_src; }
    else if (t > hi) { v = H.p + dir * hi; src = hi_src; }
    else { v = H.p + dir * t; src = -2; }
    if (kind == 0 && src != -2) return false;
    if (kind == 1 && src != -1) return false;
    if (kind == 2 && src != jsrc) return false;
    const V2 r = v - opt;
    if (kind != 1) {
        float rs = maxSpeed - margin;
        if (!(rs > 0.0f && dot(v, v) < rs * rs)) return false;
    }
    if (kind == 0) {
        if (!(dot(r, H.n) > margin)) return false;
    } else if (kind == 2) {
        const Con G = cons[jsrc];
        float d2 = det(H.n, G.n);
        float la = det(r, G.n) / d2, lb = det(H.n, r) / d2;
        if (!(la > margin && lb > margin)) return false;
    } else {
        V2 nv = v * -1.0f;
        float d2 = det(H.n, nv);
        if (!(fabsf(d2) > kEps)) return false;
        float la = det(r, nv) / d2, lb = det(H.n, r) / d2;
        if (!(la > margin && lb > margin * maxSpeed)) return false;
    }
    bool bad = false;
    for (int i = lane; i < m; i += 32) {
        if (i == h || i == jsrc) continue;
        const Con c = cons[i];
        const float d = det(right(c.n), c.p - v);
        if (i > h ? d > 0.0f : !(d < -margin)) bad = true;
    }
    if (__any_sync(kFull, bad)) return false;
    *out = v;
    return true;
}

struct WarpCounts {
    int lp3d = 0, proposed = 0, accepted = 0;
};

/* orca_tick for grid-order agent t, one warp */
template <int K>
__device__ void orca_warp(const TickArgs& a, int t, int lane, Con* cons, Con* bis, WarpCounts& wc)
{
    constexpr int MC = K + kMaxObstCons;
    const int slot = a.s_slot[t];
    if (a.active[slot] != 1) return;
    const V2 pos = a.s_pos[t];
    const V2 vel = a.s_vel[t];
    const float clr = a.s_clear[t];
    const SceneDev& sc = a.scenes[a.slot_scene ? a.slot_scene[slot] : 0];
    const float speed = a.speed[slot];
    const V2 pv = a.pref_vel[slot];
    const float maxSpeed = a.max_speed > 0.0f ? a.max_speed : speed;
    const int ncnt = a.ncnt[t];
    const int* nbr = a.nbr + (size_t)t * a.k;
    int m = 0;
    bool overflow = false;
    const float range = a.tau_o * maxSpeed + clr;
    const float rsq = range * range;
    {
        const ObstView& o = sc.ob;
        int b = 0, e = 0;
        const int* items = nullptr;
        float fx = (pos.x - o.gx0) * o.ginv, fy = (pos.y - o.gy0) * o.ginv;
        if (o.g_start && range <= o.reach && fx >= 0.0f && fy >= 0.0f && fx < (float)o.gw && fy < (float)o.gh) {
            int g = (int)fy * o.gw + (int)fx;
            b = o.g_start[g];
            e = o.g_start[g + 1];
            items = o.g_items;
        } else {
            e = o.n_verts;
        }
        for (int base = b; base < e; base += 32) {
            const int q = base + lane;
            bool emit = false;
            Con c;
            if (q < e) {
                int L = items ? items[q] : q;
                if (obstacle_in_range(o, L, pos, rsq)) emit = obstacle_constraint(o, L, pos, vel, clr, a.tau_o, &c);
            }
            const unsigned bal = __ballot_sync(kFull, emit);
            if (emit) {
                int at = m + __popc(bal & ((1u << lane) - 1u));
                if (at < MC - K) cons[at] = c;
                else overflow = true;
            }
            m += __popc(bal);
        }
        if (m > MC - K) m = MC - K;
    }
    overflow = __any_sync(kFull, overflow);
    const int nObst = m;
    if (lane < ncnt) {
        const int j = nbr[lane];
        cons[m + lane] = agent_constraint_ni(pos, vel, clr, a.s_pos[j], a.s_vel[j], a.s_clear[j], a.tau_a, a.dt,
                                             a.inv_tau_a);
    }
    m += ncnt;
    __syncwarp();
    if (overflow && lane == 0) atomicOr(&a.counters[C_ERROR], ECMG_DEV_ERR_CONSTRAINTS);

    V2 v;
    int failed = -1;
    if (a.cls || a.cls_slot) {
        const int c = a.cls_slot ? a.cls_slot[slot] : a.cls[t];
        if (c != kClsOther) {
            wc.proposed++;
            if (verify_proposal_warp(cons, m, nObst, ncnt, pv, maxSpeed, c, &v, lane)) {
                failed = m;
                wc.accepted++;
            }
        }
    }
    if (failed < 0) {
        SmemGet get{cons};
        if (a.label) {
            LpTrace tr;
            failed = lp2d_warp<SmemGet, true>(get, m, pv, maxSpeed, false, &v, &tr, lane);
            if (lane == 0) a.label[t] = (unsigned char)label_of(tr, failed, m, nObst);
        } else {
            failed = lp2d_warp<SmemGet, false>(get, m, pv, maxSpeed, false, &v, nullptr, lane);
        }
        if (failed < m) {
            lp3d_warp(cons, bis, m, nObst, maxSpeed, failed, &v, a.lp3d_fp64 != 0, lane);
            wc.lp3d++;
        }
    }

    if (lane == 0) {
        float fx = v.x - vel.x, fy = v.y - vel.y;
        V2 nv = mk(vel.x + fx * a.mass_recip * a.dt, vel.y + fy * a.mass_recip * a.dt);
        V2 npos = mk(pos.x + (nv.x * a.dt), pos.y + (nv.y * a.dt));
        a.vel[slot] = nv;
        a.pos[slot] = npos;
        if (a.rec_cnt) {
            a.rec_cnt[slot] = ncnt;
            a.rec_vorca[slot] = v;
            a.rec_fail[slot] = failed;
            a.rec_ncons[slot] = m;
            a.rec_nobst[slot] = nObst;
        }
    }
    if (a.rec_cnt && lane < a.k) a.rec_nbr[slot * a.k + lane] = lane < ncnt ? a.s_slot[nbr[lane]] : -1;
    __syncwarp(); /* cons and bis are reused by the warp's next agent */
}

/* persistent kernel, one warp per agent: a warp takes `tile` consecutive
   grid-order agents per work grab */
template <int K>
__global__ void __launch_bounds__(256) k_agents_warp(TickArgs a)
{
    constexpr int MC = K + kMaxObstCons;
    __shared__ Con s_cons[8][MC];
    __shared__ Con s_bis[8][K];
    const int n = a.counters[C_NSORTED];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int grab = a.tile > 0 ? a.tile : 1;
    WarpCounts wc;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&a.counters[C_WORK], grab);
        base = __shfl_sync(kFull, base, 0);
        if (base >= n) break;
        const int end = min(n, base + grab);
        for (int t = base; t < end; t++) orca_warp<K>(a, t, lane, s_cons[w], s_bis[w], wc);
    }
    if (lane == 0) {
        if (wc.lp3d) atomicAdd(&a.counters[C_LP3D], wc.lp3d);
        if (wc.proposed) atomicAdd(&a.counters[C_PROPOSED], wc.proposed);
        if (wc.accepted) atomicAdd(&a.counters[C_ACCEPTED], wc.accepted);
    }
}

template <int K>
__global__ void __launch_bounds__(128) k_knn(const V2* s_pos, const int* s_slot, const int* cell_start,
                                             AgentGrid g, int k, float rnb, float r2, const int* counters,
                                             int* out_ids, int* out_cnt)
{
    const int n = counters[C_NSORTED];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        Knn<K> nn;
        V2 p = s_pos[t];
        knn_grid<K>(nn, k, p, rnb, r2, s_pos, s_slot, cell_start, g);
        int slot = s_slot[t];
        out_cnt[slot] = nn.cnt;
#pragma unroll
        for (int q2 = 0; q2 < K; q2++) {
            const int q = q2 - (K - k);
            if (q >= 0) out_ids[slot * k + q] = q < nn.cnt ? (int)(unsigned)nn.key[q2] : -1;
        }
    }
}

/* ---------------------------------------------------------------------- */
static int grid_for(int n, int block, int sms, int per_sm)
{
    int g = (n + block - 1) / block;
    int cap = sms * per_sm;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

cudaError_t launch_tick(const BinArgs& b, const TickArgs& t, int max_slots, int* scan_tmp, int block, int sms,
                        cudaStream_t s, cudaStream_t s2, cudaEvent_t ev_fork, cudaEvent_t ev_join,
                        const cudaEvent_t* ev, ProposeFn propose, void* propose_user,
                        HookFn after_attract, void* after_attract_user, const KdArgs* kd)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    const unsigned evflags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
    int nb = b.total_buckets;
    cudaError_t e = cudaMemsetAsync(b.cell_count, 0, sizeof(int) * (size_t)(nb + 1), s);
    if (e != cudaSuccess) return e;
    int gb = grid_for(max_slots, 256, sms, 8);
    k_bin<<<gb, 256, 0, s>>>(b);
    e = scan(b.cell_count, (int*)b.cell_start, nb, scan_tmp, s);
    if (e != cudaSuccess) return e;
    k_scatter<<<gb, 256, 0, s>>>(b);
    /* external event nodes when captured, so that the kernel can be timed */
    if (ev) cudaEventRecordWithFlags(ev[0], s, evflags);
    if (block != 64 && block != 128 && block != 256) block = 128;
    int gk = grid_for(max_slots, 128, sms, 16);
    int per_sm = 1;
    /* the attraction kernel (second stream) and the neighbour search are
       independent: they run side by side and join before the features /
       per-agent kernels */
    e = cudaEventRecord(ev_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, ev_fork, 0);
    if (e != cudaSuccess) return e;
    int ao = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ao, k_attract, 128, 0);
    const int ga = ao > 0 && gk > sms * ao ? sms * ao : gk; /* one wave, grid-stride */
    k_attract<<<ga, 128, 0, s2>>>(t);
    if (after_attract) {
        e = after_attract(after_attract_user, s2, evflags);
        if (e != cudaSuccess) return e;
    }
    if (ev) cudaEventRecordWithFlags(ev[1], s2, evflags);
    /* the fused layout runs the neighbour search inside the per-agent kernel
       (not with a learned proposal, whose features need every list first) */
    const bool fused = t.lp_mode == 2 && !kd && !t.feat;
    if (kd) {
        /* the reference's kd-tree: build and per-member query beside the
           attraction kernel, the cache composition after it */
        e = kd_build_and_query(*kd, s, sms);
        if (e != cudaSuccess) return e;
    } else if (!fused) {
        /* one resident wave of the persistent search */
        /* two register budgets for k <= 16: 8 resident blocks per SM at
           64 registers, or 6 at 80 (no spills); the autotuner picks */
        int pn = 1;
        if (t.k <= 8 && !t.knn_wide) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pn, k_neighbors<8, 8>, 128, 0);
            k_neighbors<8, 8><<<sms * (pn > 0 ? pn : 1), 128, 0, s>>>(t);
        } else if (t.k <= 8) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pn, k_neighbors<8, 6>, 128, 0);
            k_neighbors<8, 6><<<sms * (pn > 0 ? pn : 1), 128, 0, s>>>(t);
        } else if (t.k <= 16 && !t.knn_wide) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pn, k_neighbors<16, 8>, 128, 0);
            k_neighbors<16, 8><<<sms * (pn > 0 ? pn : 1), 128, 0, s>>>(t);
        } else if (t.k <= 16) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pn, k_neighbors<16, 6>, 128, 0);
            k_neighbors<16, 6><<<sms * (pn > 0 ? pn : 1), 128, 0, s>>>(t);
        } else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pn, k_neighbors<32, 1>, 128, 0);
            k_neighbors<32, 1><<<sms * (pn > 0 ? pn : 1), 128, 0, s>>>(t);
        }
    }
    if (ev && !kd && !fused) cudaEventRecordWithFlags(ev[2], s, evflags);
    e = cudaEventRecord(ev_join, s2);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev_join, 0);
    if (e != cudaSuccess) return e;
    if (ev && fused) cudaEventRecordWithFlags(ev[2], s, evflags);
    if (kd) {
        e = kd_finish(*kd, s, sms);
        if (e != cudaSuccess) return e;
        if (ev) cudaEventRecordWithFlags(ev[2], s, evflags);
    }
    if (t.feat) {
        k_features<<<gk, 128, 0, s>>>(t);
        if (propose) {
            cudaError_t e2 = propose(propose_user, s);
            if (e2 != cudaSuccess) return e2;
        }
    }
    if (ev) cudaEventRecordWithFlags(ev[3], s, evflags);
    if (t.lp_mode == 1) {
        if (t.k <= 8) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agents_warp<8>, 256, 0);
            k_agents_warp<8><<<sms * (per_sm > 0 ? per_sm : 1), 256, 0, s>>>(t);
        } else if (t.k <= 16) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agents_warp<16>, 256, 0);
            k_agents_warp<16><<<sms * (per_sm > 0 ? per_sm : 1), 256, 0, s>>>(t);
        } else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agents_warp<32>, 256, 0);
            k_agents_warp<32><<<sms * (per_sm > 0 ? per_sm : 1), 256, 0, s>>>(t);
        }
    } else if (fused) {
        const int div = t.occ_div > 1 ? t.occ_div : 1;
        const bool full = t.cls || t.cls_slot || t.label || t.rec_cnt;
        auto go = [&](auto kern) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0);
            kern<<<sms * (per_sm / div > 0 ? per_sm / div : 1), block, 0, s>>>(t);
        };
        if (t.k <= 8) full ? go(k_agents_knn<8, true>) : go(k_agents_knn<8, false>);
        else if (t.k <= 16) full ? go(k_agents_knn<16, true>) : go(k_agents_knn<16, false>);
        else full ? go(k_agents_knn<32, true>) : go(k_agents_knn<32, false>);
    } else {
        /* persistent grid: the resident blocks per SM, divided by occ_div
           (fewer resident warps leave each more L1 for its local arrays) */
        const int div = t.occ_div > 1 ? t.occ_div : 1;
        const bool full = t.cls || t.cls_slot || t.label || t.rec_cnt;
        auto go = [&](auto kern) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, 0);
            kern<<<sms * (per_sm / div > 0 ? per_sm / div : 1), block, 0, s>>>(t);
        };
        if (t.k <= 8) full ? go(k_agents<8, true>) : go(k_agents<8, false>);
        else if (t.k <= 16) full ? go(k_agents<16, true>) : go(k_agents<16, false>);
        else full ? go(k_agents<32, true>) : go(k_agents<32, false>);
    }
    if (ev) cudaEventRecordWithFlags(ev[4], s, evflags);
    return cudaGetLastError();
}

cudaError_t launch_mark_pending(const TickArgs& t, const int* list, int n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_mark_pending<<<(n + 127) / 128, 128, 0, s>>>(t, list, n);
    return cudaGetLastError();
}

__global__ void k_mirror(const float4* __restrict__ pos, const float4* __restrict__ vel, float4* h_pos,
                         float4* h_vel, int n2, const V2* __restrict__ pos_tail, const V2* __restrict__ vel_tail,
                         V2* h_pos_tail, V2* h_vel_tail)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i], v = vel[i];
        h_pos[i] = p;
        h_vel[i] = v;
    }
    if (pos_tail && blockIdx.x == 0 && threadIdx.x == 0) {
        *h_pos_tail = *pos_tail;
        *h_vel_tail = *vel_tail;
    }
}

cudaError_t launch_mirror(const V2* pos, const V2* vel, V2* h_pos, V2* h_vel, int n, int sms, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int n2 = n / 2; /* pairs of slots as 16-byte words (the arrays are 256-byte aligned) */
    const bool odd = n & 1;
    const int g = std::max(1, std::min((n2 + 255) / 256, sms * 4));
    k_mirror<<<g, 256, 0, s>>>((const float4*)pos, (const float4*)vel, (float4*)h_pos, (float4*)h_vel, n2,
                               odd ? pos + n - 1 : nullptr, odd ? vel + n - 1 : nullptr, h_pos + n - 1, h_vel + n - 1);
    return cudaGetLastError();
}

cudaError_t launch_fixup(const TickArgs& t, const int* list, int n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const bool full = t.cls || t.cls_slot || t.label || t.rec_cnt;
    const int g = (n + 127) / 128;
    if (t.k <= 8) full ? k_fixup<8, true><<<g, 128, 0, s>>>(t, list, n) : k_fixup<8, false><<<g, 128, 0, s>>>(t, list, n);
    else if (t.k <= 16) full ? k_fixup<16, true><<<g, 128, 0, s>>>(t, list, n) : k_fixup<16, false><<<g, 128, 0, s>>>(t, list, n);
    else full ? k_fixup<32, true><<<g, 128, 0, s>>>(t, list, n) : k_fixup<32, false><<<g, 128, 0, s>>>(t, list, n);
    return cudaGetLastError();
}

cudaError_t launch_knn(const V2* pos, const unsigned char* active, int n, int k, float r, AgentGrid g,
                       int* key, int* rank, int* cell_count, int* cell_start, int* s_slot, V2* s_pos,
                       int* scan_tmp, int scan_blocks, int* out_ids, int* out_cnt, cudaStream_t s)
{
    (void)scan_blocks;
    /* the counters live behind the bucket counts: [nb+1 .. nb+1+kCounters) */
    int nb = g.ncells + 1;
    int* counters = cell_count + nb + 1;
    cudaError_t e = cudaMemsetAsync(cell_count, 0, sizeof(int) * (size_t)(nb + 1 + kCounters), s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(out_cnt, 0, sizeof(int) * (size_t)n, s);
    if (e != cudaSuccess) return e;
    /* the slot range is passed by value: the query queues no host-to-device copy */
    BinArgs b{};
    b.n_fixed = n;
    b.pos = pos;
    b.active = active;
    b.key = key;
    b.rank = rank;
    b.cell_count = cell_count;
    b.s_slot = s_slot;
    b.s_pos = s_pos;
    b.cell_start = cell_start;
    b.counters = counters;
    b.grid = g;
    b.total_buckets = nb;
    int gb = (n + 255) / 256;
    if (gb < 1) gb = 1;
    k_bin<<<gb, 256, 0, s>>>(b);
    e = scan(cell_count, cell_start, nb, scan_tmp, s);
    if (e != cudaSuccess) return e;
    k_scatter<<<gb, 256, 0, s>>>(b);
    int ga = (n + 127) / 128;
    if (ga < 1) ga = 1;
    float r2 = r * r;
    if (k <= 8) k_knn<8><<<ga, 128, 0, s>>>(s_pos, s_slot, cell_start, g, k, r, r2, counters, out_ids, out_cnt);
    else if (k <= 16) k_knn<16><<<ga, 128, 0, s>>>(s_pos, s_slot, cell_start, g, k, r, r2, counters, out_ids, out_cnt);
    else k_knn<32><<<ga, 128, 0, s>>>(s_pos, s_slot, cell_start, g, k, r, r2, counters, out_ids, out_cnt);
    return cudaGetLastError();
}

}  // namespace ecmg
