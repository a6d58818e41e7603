// split_particle on caller-owned device arrays, with no device allocation.
//
// For callers that cannot call cudaMalloc: codes whose particle arrays
// already live in device memory they manage themselves (a CUDA-Fortran or
// OpenACC port of the driver, an application-wide memory pool) and that
// must not allocate inside their time loop.  The tile counts and offsets of
// the stream compaction and the split counters live in file-scope device
// arrays of fixed size instead of a handle's buffers; every GPU that loads
// the library keeps them (about 1 MiB) until the process exits.
#include <mutex>

#include "device_common.cuh"

namespace gpat {
namespace {

// Largest parent count one call accepts: 2^26 particles, 65536 tiles of
// 1024, two int64 words per tile.
constexpr int64_t kNoAllocMaxParticles = int64_t(1) << 26;
constexpr int64_t kNoAllocTiles = kNoAllocMaxParticles / 1024;

static __device__ __align__(256) long long g_split_scratch[2 * kNoAllocTiles];
static __device__ __align__(256) DevCounters g_split_counters;

constexpr int kMaxDevices = 64;
struct DeviceSlots {
    bool ready = false;
    void *scratch = nullptr;
    DevCounters *counters = nullptr;
};
DeviceSlots g_slots[kMaxDevices];
std::mutex g_setup_mutex;

// Host code must not use the arrays' names as device addresses: on the host
// they are stand-ins.  Their device addresses are looked up once per device,
// with that device current.
int device_slots(DeviceSlots **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GPAT_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return GPAT_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSlots &s = g_slots[dev];
    if (!s.ready) {
        void *scratch = nullptr, *counters = nullptr;
        // a failed lookup leaves its error pending: clear it, so that the
        // next call does not pick it up from cudaGetLastError()
        if (cudaGetSymbolAddress(&scratch, g_split_scratch) != cudaSuccess ||
            cudaGetSymbolAddress(&counters, g_split_counters) != cudaSuccess) {
            cudaGetLastError();
            return GPAT_ERR_CUDA;
        }
        s.scratch = scratch;
        s.counters = static_cast<DevCounters *>(counters);
        s.ready = true;
    }
    *out = &s;
    return GPAT_OK;
}

}  // namespace
}  // namespace gpat

using namespace gpat;

extern "C" int gpat_split_particle_noalloc(const gpat_particles_t *dev, int64_t n,
                                           int64_t capacity, double split_ratio,
                                           double pmin_split, double p0, double pmax,
                                           void *stream, int64_t *n_out, int64_t *n_split) {
    if (!dev || !n_out || n < 0 || capacity < n) return GPAT_ERR_ARG;
    if (n > kNoAllocMaxParticles) return GPAT_ERR_ARG;   // beyond the fixed scratch
    DeviceSlots *slots = nullptr;
    int rc = device_slots(&slots);
    if (rc != GPAT_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DevParticles P;
    P.x = dev->x; P.y = dev->y; P.z = dev->z; P.p = dev->p; P.v = dev->v; P.mu = dev->mu;
    P.weight = dev->weight; P.t = dev->t; P.dt = dev->dt;
    P.split_times = dev->split_times; P.count_flag = dev->count_flag;
    P.origin = dev->origin; P.nsteps_tracked = dev->nsteps_tracked;
    P.nsteps_pushed = dev->nsteps_pushed; P.tag_injected = dev->tag_injected;
    P.tag_splitted = dev->tag_splitted; P.rng_ctr = dev->rng_ctr;
    // The counters keep the previous call's values: start them at zero.
    if (cudaMemsetAsync(slots->counters, 0, sizeof(DevCounters), s) != cudaSuccess)
        return GPAT_ERR_CUDA;
    if (launch_split_particles(P, n, capacity, split_ratio, pmin_split, p0, pmax, slots->scratch,
                               slots->counters, s) != cudaSuccess)
        return GPAT_ERR_CUDA;
    DevCounters c{};
    if (cudaMemcpyAsync(&c, slots->counters, sizeof(DevCounters), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GPAT_ERR_CUDA;
    const int64_t created = (int64_t)c.nsplit;
    *n_out = n + created;
    if (n_split) *n_split = created;
    return created < (int64_t)c.nkept ? GPAT_ERR_CAPACITY : GPAT_OK;
}
