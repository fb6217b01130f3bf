/*
 * spawn.cu -- the O(N) part of the spawn stage on the device.
 *
 * Simulator::ValidSpawnLocation (ECMAgentSimulator/Simulator.cpp:295-311)
 * scans every active agent for each candidate location, on the CPU.  Here one
 * launch tests all candidate locations of a spawn stage against the
 * device-resident agents: each thread reads one agent slot (position and
 * active flag, 9 B), finds the spawn areas whose grown box contains it (the
 * area table sits in shared memory) and tests that area's candidates with the
 * reference's expression, diff = location - position,
 * diff.x * diff.x + diff.y * diff.y < clearance * clearance (no FMA
 * contraction: the library is compiled with -fmad=false).  A candidate hit by
 * any agent is marked; marks only ever go from 0 to 1, so the result does not
 * depend on the order in which threads run.
 */
#include "ecmg_internal.h"

#include <algorithm>

namespace ecmg {

__global__ void __launch_bounds__(256) k_spawn_check(const V2* __restrict__ pos,
                                                     const unsigned char* __restrict__ active, int b, int e,
                                                     const V2* __restrict__ cand,
                                                     const SpawnAreaDev* __restrict__ areas, int n_areas,
                                                     int* __restrict__ hit)
{
    __shared__ SpawnAreaDev s_area[kSpawnMaxAreas];
    for (int i = threadIdx.x; i < n_areas; i += blockDim.x) s_area[i] = areas[i];
    __syncthreads();
    const int stride = gridDim.x * blockDim.x;
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += stride) {
        if (!active[i]) continue;
        const V2 p = pos[i];
        for (int a = 0; a < n_areas; a++) {
            const SpawnAreaDev& A = s_area[a];
            if (!(p.x >= A.x0 && p.x <= A.x1 && p.y >= A.y0 && p.y <= A.y1)) continue;
            for (int j = A.first; j < A.first + A.count; j++) {
                const V2 c = cand[j];
                const float dx = c.x - p.x, dy = c.y - p.y;
                if (dx * dx + dy * dy < A.c2) hit[j] = 1;
            }
        }
    }
}

cudaError_t launch_spawn_check(const V2* pos, const unsigned char* active, int b, int e, const V2* cand,
                               const SpawnAreaDev* areas, int n_areas, int* hit, int sms, cudaStream_t s)
{
    if (e <= b || n_areas <= 0) return cudaSuccess;
    if (n_areas > kSpawnMaxAreas) return cudaErrorInvalidValue;
    const int threads = 256;
    const long long need = ((long long)(e - b) + threads - 1) / threads;
    const int blocks = (int)std::min<long long>(need, (long long)sms * 8);
    k_spawn_check<<<blocks, threads, 0, s>>>(pos, active, b, e, cand, areas, n_areas, hit);
    return cudaGetLastError();
}

__global__ void k_spawn_place(const SpawnRec* __restrict__ rec, int n, SpawnTargets t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SpawnRec r = rec[i];
    const int s = r.slot;
    t.pos[s] = mk(r.x, r.y);
    t.vel[s] = mk(0.0f, 0.0f);
    t.pref_vel[s] = mk(0.0f, 0.0f);
    t.clear[s] = r.clr;
    t.speed[s] = r.speed;
    t.active[s] = 1;
    t.path_off[s] = r.path_off;
    t.path_len[s] = r.path_len;
    t.fail_edge[s] = -1;
}

cudaError_t launch_spawn_place(const SpawnRec* rec, int n, const SpawnTargets& t, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_spawn_place<<<(n + 127) / 128, 128, 0, s>>>(rec, n, t);
    return cudaGetLastError();
}

}  // namespace ecmg
