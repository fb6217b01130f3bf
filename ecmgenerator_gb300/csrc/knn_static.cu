/*
 * knn_static.cu -- ecmg_knn_noalloc: the stand-alone exact kNN of ecmg_knn
 * with its scratch memory in a fixed device array instead of a caller buffer.
 *
 * Who needs it: callers that may not allocate device memory when they run the
 * query -- a real-time frame loop where cudaMalloc would synchronise the
 * device and stall the frame, or a plug-in hosted by an application that owns
 * the device allocator and gives the plug-in no allocation rights.  They pass
 * their input and output arrays; everything else lives in the array below.
 *
 * The array is a file-scope __device__ variable of ECMG_KNN_STATIC_SCRATCH_BYTES
 * (16 MiB): every GPU on which the library's code is loaded holds it until the
 * process exits.  Host code must not use the variable's name as an address
 * (on the host it names a shadow object, not device memory), so the first call
 * on each device looks the device address up with cudaGetSymbolAddress while
 * that device is current and caches it; make that first call outside any
 * stream capture.  All calls share the one array and it keeps the previous
 * call's contents: the bucket counters that must start at zero are cleared by
 * every call, and calls that overlap on the GPU (different streams, or
 * different host threads on one device) race on it.
 *
 * The cached address belongs to the device's primary context, the one the
 * CUDA runtime uses.  A caller that makes another context current through the
 * driver API, or that resets the device (cudaDeviceReset) after the first
 * call, is not supported: the cached address would not be valid there.
 */
#include "../../include/ecmg.h"
#include "ecmg_internal.h"

#include <mutex>

using namespace ecmg;

static __device__ __align__(256) unsigned char g_knn_scratch[ECMG_KNN_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }
}  // namespace

extern "C" ecmg_status ecmg_knn_noalloc(const float* dev_pos, const unsigned char* dev_active, int n, int k,
                                        float radius, float min_x, float min_y, float max_x, float max_y, float cell,
                                        int* dev_out_ids, int* dev_out_count, void* stream)
{
    if (n < 0 || k < 1 || k > kMaxK || !(radius > 0.0f) || !(cell > 0.0f)) return ECMG_ERR_INVALID_ARG;
    if (n == 0) return ECMG_OK;
    if (!dev_pos || !dev_active || !dev_out_ids || !dev_out_count) return ECMG_ERR_INVALID_ARG;
    size_t need = ecmg_knn_scratch_bytes(n, min_x, min_y, max_x, max_y, cell);
    if (need == 0) return ECMG_ERR_INVALID_ARG;
    if (need > (size_t)ECMG_KNN_STATIC_SCRATCH_BYTES) return ECMG_ERR_BOUND; /* beyond the fixed array */
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ECMG_ERR_CUDA;
    void* base;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_knn_scratch) != cudaSuccess || !p) return ECMG_ERR_CUDA;
            g_addr[dev] = p;
        }
        base = g_addr[dev];
    }
    /* the same grid and partition of the scratch as ecmg_knn */
    AgentGrid g;
    if (!knn_grid_of(min_x, min_y, max_x, max_y, cell, &g)) return ECMG_ERR_INVALID_ARG;
    size_t nb = (size_t)g.ncells + 1;
    char* p = (char*)base;
    auto take = [&](size_t bytes) { char* r = p; p += a256(bytes); return r; };
    int* key = (int*)take(sizeof(int) * n);
    int* rank = (int*)take(sizeof(int) * n);
    int* s_slot = (int*)take(sizeof(int) * n);
    V2* s_pos = (V2*)take(sizeof(V2) * n);
    int* cell_count = (int*)take(sizeof(int) * (nb + 1 + kCounters));
    int* cell_start = (int*)take(sizeof(int) * (nb + 1));
    int* scan_tmp = (int*)take(sizeof(int) * (size_t)scan_tmp_ints((int)nb));
    cudaError_t e = launch_knn((const V2*)dev_pos, dev_active, n, k, radius, g, key, rank, cell_count, cell_start,
                               s_slot, s_pos, scan_tmp, 0, dev_out_ids, dev_out_count, (cudaStream_t)stream);
    return e == cudaSuccess ? ECMG_OK : ECMG_ERR_CUDA;
}
