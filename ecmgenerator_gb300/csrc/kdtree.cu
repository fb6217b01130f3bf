/*
 * kdtree.cu -- the reference's kd-tree neighbour query on the device
 * (neighbour mode ECMG_NEIGHBORS_KDTREE), results identical to
 * KDTree::Construct / KDTree::KNearestAgents_R (ECMAgentSimulator/
 * KDTree.cpp:22-202) with ORCA's neighbour cache (ORCA.h:87,100) carried from
 * agent to agent and from tick to tick.
 *
 * Build.  ConstructRecursive sorts each subtree's agents on x (even depth) or
 * y (odd depth) and takes the element at mid = lo + (hi - 1 - lo) / 2.  Equal
 * coordinates keep the order of the level above (a stable sort; libstdc++'s
 * std::sort agrees on segments of up to 16 agents, where it is an insertion
 * sort).  That order is, for depth 0, (x, agent index); for the depths after
 * it (x, y, index) and (y, x, index).  So the build sorts the members once
 * into three lists, X0 = (x, index), X = (x, y, index), Y = (y, x, index), by
 * stable LSD radix passes, and then walks the levels: the list of the level's
 * axis is already sorted inside every segment, its element at mid is the node,
 * and the other list is partitioned stably into (left, node, right) with one
 * scan of left / right flags.  Segments are position ranges shared by both
 * lists.  O(N) work per level.
 *
 * Query.  One thread per member replays KNearestAgents_R with an explicit
 * stack.  The reference does not clear the cache between agents: slots that a
 * query does not overwrite keep the previous agent's entries, and entries
 * move between slots.  The thread therefore starts from the symbolic cache
 * (-1, -2, ..., -k) = "previous agent's slot q" and ends with a map: each
 * slot either an agent or a previous slot.  Maps compose associatively; the
 * composition over the querying agents in index order (members still active
 * after the attraction stage) runs as a warp per block of 1024 slots, one
 * warp over the block results, and a resolving pass -- the last agent's list
 * is the cache the next tick starts from.
 */
#include "ecmg_internal.h"

#include <cfloat>

namespace ecmg {

namespace {

constexpr int kRsThreads = 256, kRsItems = 16, kRsTile = kRsThreads * kRsItems;
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;
constexpr int kComposeSlots = 1024;

__device__ __forceinline__ unsigned order_key(float f)
{
    unsigned u = __float_as_uint(f);
    if (u == 0x80000000u) u = 0u; /* -0 == +0 for operator< */
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* ---- exclusive scan (in place), T = int or unsigned long long ---------- */
template <typename T>
__device__ T block_excl_scan(T v, T* total)
{
    __shared__ T warp_sum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    if (w == 0) {
        T s = lane < kScanThreads / 32 ? warp_sum[lane] : (T)0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanThreads / 32) warp_sum[lane] = s;
    }
    __syncthreads();
    const T before = (w > 0 ? warp_sum[w - 1] : (T)0) + x - v;
    if (total) *total = warp_sum[kScanThreads / 32 - 1];
    __syncthreads();
    return before;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const T* __restrict__ in, int n, T* __restrict__ sums)
{
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
        if (base + i < n) s += in[base + i];
    T tot;
    block_excl_scan<T>(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

/* one block of 1024 threads: exclusive scan of nb <= 8192 block sums */
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_top(T* sums, int nb)
{
    __shared__ T ws[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T v[8];
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int j = threadIdx.x * 8 + i;
        v[i] = j < nb ? sums[j] : (T)0;
        s += v[i];
    }
    T x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        T t = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    T run = (w > 0 ? ws[w - 1] : (T)0) + x - s;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int j = threadIdx.x * 8 + i;
        if (j < nb) sums[j] = run;
        run += v[i];
    }
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_down(T* __restrict__ data, int n, const T* __restrict__ sums)
{
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    T v[kScanItems];
    T s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = base + i < n ? data[base + i] : (T)0;
        s += v[i];
    }
    T run = block_excl_scan<T>(s, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) data[base + i] = run;
        run += v[i];
    }
}

template <typename T>
cudaError_t scan_excl(T* data, int n, T* tmp, cudaStream_t s)
{
    const int nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) return cudaSuccess;
    if (nb > 8192) return cudaErrorInvalidValue;
    k_scan_reduce<T><<<nb, kScanThreads, 0, s>>>(data, n, tmp);
    k_scan_top<T><<<1, 1024, 0, s>>>(tmp, nb);
    k_scan_down<T><<<nb, kScanThreads, 0, s>>>(data, n, tmp);
    return cudaGetLastError();
}

/* ---- stable LSD radix sort of (key, value) pairs, 8-bit digits ---------- */
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const unsigned* __restrict__ keys, const int* __restrict__ n_ptr,
                                                        int shift, int* __restrict__ hist, int nblk)
{
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int n = *n_ptr;
    const int base = blockIdx.x * kRsTile;
#pragma unroll 4
    for (int i = 0; i < kRsItems; i++) {
        const int idx = base + i * kRsThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

/* elements of a tile are placed in tile order, round by round (256 per
   round, in thread order): rank among equal digits = warps before + lanes
   before, so the pass is stable */
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const unsigned* __restrict__ kin, const int* __restrict__ vin,
                                                           unsigned* __restrict__ kout, int* __restrict__ vout,
                                                           const int* __restrict__ n_ptr, int shift,
                                                           const int* __restrict__ offs, int nblk)
{
    __shared__ int base[256];
    __shared__ int wc[kRsThreads / 32][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = *n_ptr;
    base[threadIdx.x] = offs[threadIdx.x * nblk + blockIdx.x];
    const int t0 = blockIdx.x * kRsTile;
    for (int r = 0; r < kRsItems; r++) {
#pragma unroll
        for (int q = 0; q < kRsThreads / 32; q++) wc[q][threadIdx.x] = 0;
        __syncthreads();
        const int idx = t0 + r * kRsThreads + threadIdx.x;
        const bool valid = idx < n;
        const unsigned key = valid ? kin[idx] : 0u;
        const int d = valid ? (int)((key >> shift) & 255u) : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wc[w][d] = __popc(peers);
        __syncthreads();
        {
            int run = base[threadIdx.x];
#pragma unroll
            for (int q = 0; q < kRsThreads / 32; q++) {
                const int c = wc[q][threadIdx.x];
                wc[q][threadIdx.x] = run;
                run += c;
            }
            base[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            const int pos = wc[w][d] + rank;
            kout[pos] = key;
            vout[pos] = vin[idx];
        }
        __syncthreads();
    }
}

/* sorts keys[0, n) with their values; n is read on the device; the result
   ends in (keys, vals) after the four passes */
cudaError_t radix_sort(unsigned* keys, int* vals, unsigned* ktmp, int* vtmp, const int* n_ptr, int cap, int* hist,
                       int* scan_tmp, cudaStream_t s)
{
    const int nblk = (cap + kRsTile - 1) / kRsTile;
    unsigned* ka = keys;
    int* va = vals;
    unsigned* kb = ktmp;
    int* vb = vtmp;
    for (int shift = 0; shift < 32; shift += 8) {
        k_rs_hist<<<nblk, kRsThreads, 0, s>>>(ka, n_ptr, shift, hist, nblk);
        cudaError_t e = scan_excl<int>(hist, 256 * nblk, scan_tmp, s);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<nblk, kRsThreads, 0, s>>>(ka, va, kb, vb, n_ptr, shift, hist, nblk);
        unsigned* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
    }
    return cudaGetLastError();
}

/* ---- members, keys and lists ------------------------------------------- */
__global__ void k_kd_mark(KdArgs a)
{
    const int n = a.counters[C_NSORTED];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) a.mark[a.s_slot[t]] = 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.n_dev[0] = n;
        /* KDTree.cpp:47: ceil(log2(size + 1) - 1) = bit length of size - 1 */
        a.n_dev[1] = n > 0 ? 31 - __clz(n) : -1;
    }
}

__global__ void k_kd_flag(KdArgs a, int* flags)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.max_slots; i += gridDim.x * blockDim.x)
        flags[i] = a.mark[i];
}

__global__ void k_kd_compact(KdArgs a, const int* flags, int* ids)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.max_slots; i += gridDim.x * blockDim.x)
        if (a.mark[i]) ids[flags[i]] = i;
}

__global__ void k_kd_keys(KdArgs a, const int* ids, int axis, unsigned* keys, int* vals)
{
    const int n = a.n_dev[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int id = ids[i];
        const V2 p = a.pos[id];
        keys[i] = order_key(axis ? p.y : p.x);
        vals[i] = id;
    }
}

__global__ void k_kd_seg_init(KdArgs a)
{
    const int n = a.n_dev[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.cap; i += gridDim.x * blockDim.x) {
        a.seg_lo[i] = 0;
        a.seg_hi[i] = i < n ? n : 0;
        a.seg_node[i] = 0;
    }
}

/* ---- one level of ConstructRecursive ------------------------------------ */
__global__ void k_kd_side(KdArgs a, const int* A)
{
    const int n = a.n_dev[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int lo = a.seg_lo[i], hi = a.seg_hi[i];
        if (lo >= hi) continue;
        const int mid = lo + (hi - 1 - lo) / 2;
        const int id = A[i];
        a.side[id] = i < mid ? 0 : (i == mid ? 1 : 2);
        if (i == mid) a.tree[a.seg_node[i]] = id;
    }
}

__global__ void k_kd_lrflags(KdArgs a, const int* B)
{
    const int n = a.n_dev[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.cap; i += gridDim.x * blockDim.x) {
        unsigned long long f = 0;
        if (i < n && a.seg_lo[i] < a.seg_hi[i]) {
            const int s = a.side[B[i]];
            f = (s == 0 ? 1ull : 0ull) | (s == 2 ? (1ull << 32) : 0ull);
        }
        a.flags[i] = f;
    }
}

/* stable partition of B's segments into (left, node, right); update_seg
   also moves every position to its child segment (after the last use of
   the level's segments) */
__global__ void k_kd_partition(KdArgs a, const int* B, int* Bout, int update_seg)
{
    const int n = a.n_dev[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int lo = a.seg_lo[i], hi = a.seg_hi[i];
        if (lo >= hi) {
            Bout[i] = B[i];
            continue;
        }
        const int mid = lo + (hi - 1 - lo) / 2;
        const unsigned long long f = a.flags[i], f0 = a.flags[lo];
        const int id = B[i];
        const int s = a.side[id];
        int pos;
        if (s == 0) pos = lo + (int)((unsigned)f - (unsigned)f0);
        else if (s == 1) pos = mid;
        else pos = mid + 1 + (int)((unsigned)(f >> 32) - (unsigned)(f0 >> 32));
        Bout[pos] = id;
        if (update_seg) {
            const int node = a.seg_node[i];
            if (i < mid) {
                a.seg_hi[i] = mid;
                a.seg_node[i] = 2 * node + 1;
            } else if (i > mid) {
                a.seg_lo[i] = mid + 1;
                a.seg_node[i] = 2 * node + 2;
            } else {
                a.seg_lo[i] = hi;
            }
        }
    }
}

/* positions in tree order (one dependent load per visit in the query) */
__global__ void k_kd_tree_pos(KdArgs a)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.tree_cap; i += gridDim.x * blockDim.x) {
        const int id = a.tree[i];
        a.tree_pos[i] = id >= 0 ? a.pos[id] : mk(0.0f, 0.0f);
    }
}

/* ---- KNearestAgents_R (KDTree.cpp:98-202) with a symbolic cache ---------- */
__global__ void __launch_bounds__(128) k_kd_query(KdArgs a, const int* members)
{
    const int n = a.n_dev[0];
    const int max_depth = a.n_dev[1];
    const int k = a.k;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int agent = members[i];
        const V2 target = a.pos[agent];
        int ni[kMaxK];
        float nd[kMaxK];
        for (int q = 0; q < k; q++) {
            ni[q] = -(q + 1); /* the previous agent's slot q */
            nd[q] = FLT_MAX;  /* Utility::MAX_FLOAT */
        }
        int kfound = 0;
        /* frames: node and stage (0 visit, 1 first child done, 2 both),
           and the least |x - target.x|, |y - target.y| of the subtree's
           region known from the split planes above it */
        /* frame j holds a node of depth j: node | stage << 28 */
        int st[kKdMaxDepth + 2];
        float2 stb[kKdMaxDepth + 2];
        st[0] = 0;
        stb[0] = make_float2(0.0f, 0.0f);
        int sp = 1;
        while (sp > 0) {
            const int node = st[sp - 1] & 0x0fffffff;
            const int depth = sp - 1;
            const int stage = st[sp - 1] >> 28;
            if (stage == 0) {
                if (depth > max_depth) {
                    sp--;
                    continue;
                }
                /* the node's slot and its position (tree order, loaded
                   side by side) */
                const int cur = a.tree[node];
                const V2 cp = a.tree_pos[node];
                if (cur == -1) {
                    sp--;
                    continue;
                }
                /* Once k are found, visiting a node changes nothing unless
                   d < nd[0]; every node of this subtree has
                   d >= bx^2 + by^2 (rounding is monotonic), so when that
                   bound reaches nd[0] the whole subtree is visited by the
                   reference without effect and is skipped here. */
                if (kfound == k) {
                    const float bx = stb[sp - 1].x, by = stb[sp - 1].y;
                    if (bx * bx + by * by >= nd[0]) {
                        sp--;
                        continue;
                    }
                }
                const float dx = cp.x - target.x, dy = cp.y - target.y;
                const float d = dx * dx + dy * dy;
                if (kfound < k && d > 1e-4f) {
                    ni[kfound] = cur;
                    nd[kfound] = d;
                    kfound++;
                    if (kfound == k) {
                        float largest = d;
                        int li = k - 1;
                        for (int q = 0; q < k - 1; q++)
                            if (nd[q] > largest) {
                                largest = nd[q];
                                li = q;
                            }
                        nd[0] = largest;
                        ni[0] = ni[li];
                        nd[li] = d;
                        ni[li] = cur;
                    }
                } else {
                    kfound = k;
                    if (d < nd[0] && d > 1e-4f) {
                        nd[0] = d;
                        ni[0] = cur;
                        float largest = d;
                        int li = 0;
                        for (int q = 1; q < k; q++)
                            if (nd[q] > largest) {
                                largest = nd[q];
                                li = q;
                            }
                        nd[0] = largest;
                        ni[0] = ni[li];
                        nd[li] = d;
                        ni[li] = cur;
                    }
                }
                const float cv = (depth & 1) == 0 ? cp.x : cp.y;
                const float tv = (depth & 1) == 0 ? target.x : target.y;
                st[sp - 1] = node | (1 << 28);
                st[sp] = tv < cv ? 2 * node + 1 : 2 * node + 2;
                stb[sp] = stb[sp - 1]; /* the near side: no new bound */
                sp++;
            } else if (stage == 1) {
                const V2 cp = a.tree_pos[node];
                const float cv = (depth & 1) == 0 ? cp.x : cp.y;
                const float tv = (depth & 1) == 0 ? target.x : target.y;
                const float db = tv - cv;
                if (db * db < nd[k - 1]) {
                    st[sp - 1] = node | (2 << 28);
                    st[sp] = tv < cv ? 2 * node + 2 : 2 * node + 1;
                    /* the far side: at least |db| away along this axis */
                    float2 b = stb[sp - 1];
                    if ((depth & 1) == 0) b.x = fmaxf(b.x, fabsf(db));
                    else b.y = fmaxf(b.y, fabsf(db));
                    stb[sp] = b;
                    sp++;
                } else {
                    sp--;
                }
            } else {
                sp--;
            }
        }
        int* m = a.map + (size_t)agent * k;
        for (int q = 0; q < k; q++) m[q] = ni[q];
        a.kfound[agent] = kfound;
    }
}

/* ---- composition of the maps in slot order ------------------------------ */
__device__ __forceinline__ bool querying(const KdArgs& a, int s)
{
    return a.mark[s] && a.active[s];
}

/* one warp per block of kComposeSlots slots, lane q = cache slot q: local
   prefix maps (in place) and the block's map.  The rows of 32 slots at a
   time are staged in shared memory, so that the sequential chain runs on
   shared memory. */
__global__ void __launch_bounds__(32) k_kd_compose_local(KdArgs a)
{
    __shared__ int rows[32][kMaxK];
    __shared__ int use[32];
    const int q = threadIdx.x;
    const int k = a.k;
    const int last = a.counters[C_LAST];
    const int s0 = blockIdx.x * kComposeSlots;
    const int s1 = min(s0 + kComposeSlots, last + 1);
    int cur = -(q + 1);
    for (int c0 = s0; c0 < s1; c0 += 32) {
        const int cn = min(32, s1 - c0);
        use[q] = q < cn && querying(a, c0 + q);
        __syncwarp();
#pragma unroll 8
        for (int j = 0; j < cn; j++)
            if (use[j] && q < k) rows[j][q] = a.map[(size_t)(c0 + j) * k + q];
        __syncwarp();
        for (int j = 0; j < cn; j++) {
            if (!use[j]) continue;
            int v = q < k ? rows[j][q] : -(q + 1);
            const int src = v < 0 ? -v - 1 : q;
            const int got = __shfl_sync(0xffffffffu, cur, src);
            if (v < 0) v = got;
            cur = v;
            if (q < k) rows[j][q] = v;
        }
        __syncwarp();
#pragma unroll 8
        for (int j = 0; j < cn; j++)
            if (use[j] && q < k) a.map[(size_t)(c0 + j) * k + q] = rows[j][q];
        __syncwarp();
    }
    if (q < k) a.agg[(size_t)blockIdx.x * k + q] = cur;
}

/* one warp: the list each block starts from, and the cache the next tick
   starts from (block maps staged 32 at a time) */
__global__ void __launch_bounds__(32) k_kd_compose_top(KdArgs a, int nblk)
{
    __shared__ int rows[32][kMaxK];
    const int q = threadIdx.x;
    const int k = a.k;
    const int last = a.counters[C_LAST];
    const int used = last < 0 ? 0 : min(nblk, last / kComposeSlots + 1);
    int prev = q < k ? a.cache[q] : 0;
    for (int c0 = 0; c0 < used; c0 += 32) {
        const int cn = min(32, used - c0);
        for (int j = 0; j < cn; j++)
            if (q < k) rows[j][q] = a.agg[(size_t)(c0 + j) * k + q];
        __syncwarp();
        for (int j = 0; j < cn; j++) {
            if (q < k) a.prev_in[(size_t)(c0 + j) * k + q] = prev;
            const int v = q < k ? rows[j][q] : -(q + 1);
            const int src = v < 0 ? -v - 1 : q;
            const int got = __shfl_sync(0xffffffffu, prev, src);
            prev = v < 0 ? got : v;
        }
        __syncwarp();
    }
    if (q < k) a.cache[q] = prev;
}

/* grid index of every slot (members), -(slot + 1) for the others */
__global__ void k_kd_gidx(KdArgs a)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < a.max_slots; s += gridDim.x * blockDim.x)
        a.iscan[s] = a.mark[s] ? a.cell_start[a.slot_bucket[s]] + a.slot_rank[s] : -(s + 1);
}

/* final lists -> the per-agent kernel's inputs (grid order): a neighbour in
   this tick's grid by its grid index, any other slot as -(slot + 1) */
__global__ void k_kd_emit(KdArgs a)
{
    const int k = a.k;
    const int last = a.counters[C_LAST];
    const int* gidx = a.iscan;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s <= last; s += gridDim.x * blockDim.x) {
        if (!querying(a, s)) continue;
        const int t = gidx[s];
        const int b = s / kComposeSlots;
        const int cnt = a.kfound[s];
        int* out = a.nbr + (size_t)t * k;
        for (int q = 0; q < cnt; q++) {
            int v = a.map[(size_t)s * k + q];
            if (v < 0) v = a.prev_in[(size_t)b * k + (-v - 1)];
            out[q] = gidx[v];
        }
        a.ncnt[t] = cnt;
    }
}

int grid_n(int n, int threads, int sms)
{
    const long long need = ((long long)n + threads - 1) / threads;
    const long long cap = (long long)sms * 16;
    return (int)std::max(1LL, std::min(need, cap));
}

}  // namespace

int kd_compose_blocks(int max_slots) { return (max_slots + kComposeSlots - 1) / kComposeSlots; }
int kd_hist_ints(int cap) { return 256 * ((cap + kRsTile - 1) / kRsTile); }
int kd_scan_tmp(int n) { return (n + kScanTile - 1) / kScanTile + 1; }

/* the build and the per-member maps, on s (beside the attraction kernel) */
cudaError_t kd_build_and_query(const KdArgs& a, cudaStream_t s, int sms)
{
    cudaError_t e = cudaMemsetAsync(a.mark, 0, (size_t)a.max_slots, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.tree, 0xff, sizeof(int) * (size_t)a.tree_cap, s);
    if (e != cudaSuccess) return e;
    const int gs = grid_n(a.max_slots, 256, sms), gc = grid_n(a.cap, 256, sms);
    k_kd_mark<<<gc, 256, 0, s>>>(a);
    /* members in slot order */
    k_kd_flag<<<gs, 256, 0, s>>>(a, a.iscan);
    e = scan_excl<int>(a.iscan, a.max_slots, a.scan_tmp32, s);
    if (e != cudaSuccess) return e;
    k_kd_compact<<<gs, 256, 0, s>>>(a, a.iscan, a.ids0);
    /* X0 = (x, index); Y = (y, x, index) sorted from X0 */
    k_kd_keys<<<gc, 256, 0, s>>>(a, a.ids0, 0, a.keys, a.X0);
    e = radix_sort(a.keys, a.X0, a.ktmp, a.vtmp, a.n_dev, a.cap, a.hist, a.scan_tmp32, s);
    if (e != cudaSuccess) return e;
    k_kd_keys<<<gc, 256, 0, s>>>(a, a.X0, 1, a.keys, a.Y[0]);
    e = radix_sort(a.keys, a.Y[0], a.ktmp, a.vtmp, a.n_dev, a.cap, a.hist, a.scan_tmp32, s);
    if (e != cudaSuccess) return e;
    /* X = (x, y, index) sorted from (y, index) */
    k_kd_keys<<<gc, 256, 0, s>>>(a, a.ids0, 1, a.keys, a.X[1]);
    e = radix_sort(a.keys, a.X[1], a.ktmp, a.vtmp, a.n_dev, a.cap, a.hist, a.scan_tmp32, s);
    if (e != cudaSuccess) return e;
    k_kd_keys<<<gc, 256, 0, s>>>(a, a.X[1], 0, a.keys, a.X[0]);
    e = radix_sort(a.keys, a.X[0], a.ktmp, a.vtmp, a.n_dev, a.cap, a.hist, a.scan_tmp32, s);
    if (e != cudaSuccess) return e;
    k_kd_seg_init<<<gc, 256, 0, s>>>(a);
    /* level 0 splits on X0 and partitions X and Y; then Y / X alternate */
    int xi = 0, yi = 0;
    for (int lv = 0; lv < a.levels; lv++) {
        if (lv == 0) {
            k_kd_side<<<gc, 256, 0, s>>>(a, a.X0);
            k_kd_lrflags<<<gc, 256, 0, s>>>(a, a.X[xi]);
            e = scan_excl<unsigned long long>(a.flags, a.cap, a.scan_tmp64, s);
            if (e != cudaSuccess) return e;
            k_kd_partition<<<gc, 256, 0, s>>>(a, a.X[xi], a.X[xi ^ 1], 0);
            xi ^= 1;
            k_kd_lrflags<<<gc, 256, 0, s>>>(a, a.Y[yi]);
            e = scan_excl<unsigned long long>(a.flags, a.cap, a.scan_tmp64, s);
            if (e != cudaSuccess) return e;
            k_kd_partition<<<gc, 256, 0, s>>>(a, a.Y[yi], a.Y[yi ^ 1], 1);
            yi ^= 1;
        } else {
            const bool on_y = (lv & 1) != 0;
            const int* A = on_y ? a.Y[yi] : a.X[xi];
            k_kd_side<<<gc, 256, 0, s>>>(a, A);
            if (lv + 1 < a.levels) {
                const int* B = on_y ? a.X[xi] : a.Y[yi];
                int* Bout = on_y ? a.X[xi ^ 1] : a.Y[yi ^ 1];
                k_kd_lrflags<<<gc, 256, 0, s>>>(a, B);
                e = scan_excl<unsigned long long>(a.flags, a.cap, a.scan_tmp64, s);
                if (e != cudaSuccess) return e;
                k_kd_partition<<<gc, 256, 0, s>>>(a, B, Bout, 1);
                if (on_y) xi ^= 1;
                else yi ^= 1;
            }
        }
    }
    /* queries in grid order: the agents of a warp are neighbours, so their
       traversals share nodes in cache */
    k_kd_tree_pos<<<grid_n(a.tree_cap, 256, sms), 256, 0, s>>>(a);
    k_kd_query<<<grid_n(a.cap, 128, sms), 128, 0, s>>>(a, a.s_slot);
    return cudaGetLastError();
}

/* after the attraction kernel: composition in slot order, then the inputs
   of the per-agent kernel */
cudaError_t kd_finish(const KdArgs& a, cudaStream_t s, int sms)
{
    const int nblk = kd_compose_blocks(a.max_slots);
    k_kd_compose_local<<<nblk, 32, 0, s>>>(a);
    k_kd_compose_top<<<1, 32, 0, s>>>(a, nblk);
    k_kd_gidx<<<grid_n(a.max_slots, 256, sms), 256, 0, s>>>(a);
    k_kd_emit<<<grid_n(a.max_slots, 256, sms), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace ecmg
