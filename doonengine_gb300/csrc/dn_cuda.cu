/*
 * dn_cuda.cu -- CUDA kernels for sm_103a and the C ABI of include/dn_cuda.h.
 *
 * Device layout of one map (struct DNgpuVolume):
 *   tiles   tword[t] = state << 30 | record slot   (state 0 absent, 1 unloaded, 2 loaded)
 *           treq / tvis / ttouch (bytes), tlast (lastUsed), tpend / tpendSlot (host ops of a sync)
 *   records rec[slot]: 128-B ChunkRec (512-bit occupancy mask, partial counts, voxel count,
 *           position, pool base, material set), nsamples[slot]
 *   pool    vox[i] (uint2: normal word, linear albedo word), diff[i] / spec[i] (float4, FP32)
 *   frame   reqs[] ((tile << 4) | group), lightOut[] (scratch: new lighting per request lane)
 * Kernels per frame: k_draw (primary rays); k_pack_stage (or k_sync_stage for records packed on the host)
 * + k_compact (DN_sync_gpu); k_mark_opaque + k_light_tables + k_light_packet + k_light_diffuse (or
 * k_light_stream) + k_commit (DN_update_lighting).
 */
#include "dn_internal.cuh"
#include "dn_light_stream.cuh"
#include "dn_light_packet.cuh"
#include <stdio.h>
#include <string.h>
#include <stdlib.h>
#include <new>
#include <mutex>
#include <vector>
#include <stdarg.h>

using namespace dn;

static_assert(sizeof(dn_material) == 32, "material layout");
static_assert(sizeof(Material) == 32, "material layout");
static_assert(sizeof(ChunkRec) == 128, "record layout");
static_assert(sizeof(dn_chunk_record) == 96, "record layout");

// ------------------------------------------------------------------ errors

static thread_local char t_err[512] = "";

int dn_set_err(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
    return code;
}


extern "C" const char* dn_cuda_last_error(void) { return t_err; }

extern "C" const char* dn_cuda_error_string(int code)
{
    switch (code) {
    case DN_CUDA_OK: return "ok";
    case DN_CUDA_ERR_ARG: return "invalid argument";
    case DN_CUDA_ERR_NOMEM: return "out of memory";
    case DN_CUDA_ERR_LAUNCH: return "CUDA runtime error";
    case DN_CUDA_ERR_DEVICE: return "no usable CUDA device";
    case DN_CUDA_ERR_KERNEL: return "kernel reported an error";
    case DN_CUDA_ERR_CAPACITY: return "capacity exceeded";
    default: return "unknown error";
    }
}

int g_device = -1;
int g_numSMs = 0;
bool g_asyncAlloc = false;
// pinned host blocks kept by restored volumes for their next eviction, and the cap on their sum
// (DN_PINNED_RETAIN_GB, default 64 GiB): within it a map's evictions after the first pin nothing
// the pinned host memory evictions copy into: 64 MiB slabs, pinned once and reused by every volume.  A slab's
// event marks the end of the last copy that read it (a restore), so that the next eviction writing it waits
// for that copy on the device, never on the host.
static const size_t HOST_SLAB = 64ull << 20;
struct HostSlab { unsigned char* p; cudaEvent_t lastRead; };
static std::mutex g_slabMutex;
static std::vector<HostSlab> g_slabs;
static std::vector<uint32_t> g_freeSlabs;
// Evictions and restores copy on streams of their own, so that their copies overlap the kernels of other
// maps; evictions (device to host) and restores (host to device) on separate streams, so that a restore
// never queues behind evictions and the two directions overlap.  Pool memory an eviction frees becomes
// reusable by a restore once the eviction's frees have run (the stream-ordered allocator tracks that).
static cudaStream_t g_copyStream = nullptr;      // evictions
static cudaStream_t g_restoreStream = nullptr;   // restores
static int g_copyStreamDevice = -1;
unsigned long long g_launches = 0;
unsigned long long g_allocs = 0;
static unsigned long long g_generation = 0;

// a process-wide unique generation: graphs keyed on (volume, generation) never match a volume that was
// freed and re-created at the same address, nor arrays that were reallocated
void dn_new_generation(DNgpuVolume* g) { g->gen = __atomic_add_fetch(&g_generation, 1ull, __ATOMIC_RELAXED); }

extern "C" uint64_t dn_cuda_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
extern "C" uint64_t dn_cuda_alloc_count(void) { return __atomic_load_n(&g_allocs, __ATOMIC_RELAXED); }

// lighting kernel selection and stream batch threshold (DN_LIGHT_KERNEL=1 per-lane ray streams, 2 warp packets
// of ray fans; DN_STREAM_BATCH lanes, 1..32), read once at init
int g_lightKernel = 2;
uint32_t g_streamBatch = 24;
uint32_t g_packetBatch = 12;   // lanes with an ended segment before the packet kernel shades (measured best)

static void noalloc_forget(void);

extern "C" int dn_cuda_init(int device)
{
    if (const char* e = getenv("DN_LIGHT_KERNEL")) g_lightKernel = atoi(e) == 1 ? 1 : 2;
    if (const char* e = getenv("DN_STREAM_BATCH")) {
        int b = atoi(e);
        g_streamBatch = (uint32_t)(b < 1 ? 1 : (b > 32 ? 32 : b));
    }
    if (const char* e = getenv("DN_PACKET_BATCH")) {
        int b = atoi(e);
        g_packetBatch = (uint32_t)(b < 1 ? 1 : (b > 32 ? 32 : b));
    }
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return dn_set_err(DN_CUDA_ERR_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    }
    if (device < 0) CK(cudaGetDevice(&device));
    if (device >= n) return dn_set_err(DN_CUDA_ERR_ARG, "device %d of %d", device, n);
    CK(cudaSetDevice(device));
    CK(cudaFree(0));
    CK(cudaDeviceGetAttribute(&g_numSMs, cudaDevAttrMultiProcessorCount, device));
    // stream-ordered allocation for volume arrays that come and go with eviction: the device's default pool
    // keeps what it frees (release threshold unlimited), so a restore reuses an evicted map's memory
    // without returning to the driver, and a free does not wait for the whole device
    int pools = 0;
    g_asyncAlloc = false;
    if (cudaDeviceGetAttribute(&pools, cudaDevAttrMemoryPoolsSupported, device) == cudaSuccess && pools) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = ~0ull;
            if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess) g_asyncAlloc = true;
        }
    }
    cudaGetLastError();
    g_device = device;
    noalloc_forget();
    return DN_CUDA_OK;
}

extern "C" void dn_cuda_shutdown(void) { g_device = -1; noalloc_forget(); }


uint32_t vol_array_bit(DNgpuVolume* g, const void* field)
{
    const void* fields[] = {&g->tword, &g->treq, &g->tvis, &g->ttouch, &g->tbits, &g->tlast, &g->tpend, &g->tpendSlot,
                            &g->rec, &g->nsamples, &g->vox, &g->diff, &g->spec, &g->reqs, &g->st, &g->dtab,
                            &g->lightOut, &g->dstage, &g->dimg, &g->dhit, &g->dface};
    for (uint32_t i = 0; i < sizeof(fields) / sizeof(fields[0]); i++)
        if (fields[i] == field) return 1u << i;
    return 0u;
}

static int alloc_tiles(DNgpuVolume* g)
{
    uint64_t n = g->ntiles;
    int rc;
    dn_new_generation(g);
    if ((rc = valloc(g, g->tword, n)) || (rc = valloc(g, g->treq, n)) || (rc = valloc(g, g->tvis, n)) ||
        (rc = valloc(g, g->tbits, (n + 31) / 32 * 2)) ||
        (rc = valloc(g, g->ttouch, n)) || (rc = valloc(g, g->tlast, n)) || (rc = valloc(g, g->tpend, n)) ||
        (rc = valloc(g, g->tpendSlot, n)))
        return rc;
    CK(cudaMemsetAsync(g->tword, 0, n * 4, g->stream));
    CK(cudaMemsetAsync(g->tbits, 0, (n + 31) / 32 * 8, g->stream));
    CK(cudaMemsetAsync(g->treq, 0, n, g->stream));
    CK(cudaMemsetAsync(g->tvis, 0, n, g->stream));
    CK(cudaMemsetAsync(g->ttouch, 0, n, g->stream));
    CK(cudaMemsetAsync(g->tlast, 0, n * 4, g->stream));
    CK(cudaMemsetAsync(g->tpend, 0, n * 4, g->stream));
    return DN_CUDA_OK;
}

static void free_tiles(DNgpuVolume* g, cudaStream_t s = nullptr)
{
    vfree(g, g->tword, s); vfree(g, g->tbits, s); vfree(g, g->treq, s); vfree(g, g->tvis, s); vfree(g, g->ttouch, s);
    vfree(g, g->tlast, s); vfree(g, g->tpend, s); vfree(g, g->tpendSlot, s);
}

extern "C" void dn_cuda_map_destroy(DNgpuVolume* g)
{
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->batch) dn_cuda_batch_remove(g->batch, g);
    if (g->stream) cudaStreamSynchronize(g->stream);
    free_tiles(g);
    vfree(g, g->rec); vfree(g, g->nsamples); vfree(g, g->vox); vfree(g, g->diff); vfree(g, g->spec);
    vfree(g, g->reqs); vfree(g, g->lightOut); vfree(g, g->st); vfree(g, g->dtab); vfree(g, g->dstage);
    vfree(g, g->dimg); vfree(g, g->dhit); vfree(g, g->dface);
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (int k = 0; k < 2; k++)
        if (g->hstage[k]) cudaFreeHost(g->hstage[k]);
    if (g->hst) cudaFreeHost(g->hst);
    if (g->evicted) {
        // an evicted volume's slabs go back to the pool (no copy reads them any more)
        std::lock_guard<std::mutex> lock(g_slabMutex);
        for (uint32_t i = 0; i < g->evictedSlabs; i++) g_freeSlabs.push_back(g->evicted[i]);
        free(g->evicted);
    }
    for (int k = 0; k < 2; k++)
        if (g->stageFree[k]) cudaEventDestroy(g->stageFree[k]);
    if (g->copyDone) cudaEventDestroy(g->copyDone);
    if (g->ownStream) cudaStreamDestroy(g->ownStream);
    delete g;
}

static int reserve_requests(DNgpuVolume* g, uint64_t cap)
{
    if (cap <= g->reqCap) return DN_CUDA_OK;
    uint64_t nc = g->reqCap ? g->reqCap : 1024;
    while (nc < cap) nc *= 2;
    CK(cudaStreamSynchronize(g->stream));
    vfree(g, g->reqs); vfree(g, g->lightOut);
    dn_new_generation(g);
    int rc;
    if ((rc = valloc(g, g->reqs, nc)) || (rc = valloc(g, g->lightOut, nc * 64))) { g->reqCap = 0; return rc; }
    g->reqCap = nc;
    // the old request list is gone: nothing may be lit from it
    if (g->st) CK(cudaMemsetAsync(&g->st->w[ST_REQ], 0, 4, g->stream));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_map_create(uint32_t sx, uint32_t sy, uint32_t sz, uint32_t slotCap, uint64_t voxelCap,
                                  DNgpuVolume** out)
{
    if (!out) return dn_set_err(DN_CUDA_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (g_device < 0) return dn_set_err(DN_CUDA_ERR_DEVICE, "dn_cuda_init was not called");
    uint64_t n = (uint64_t)sx * sy * sz;
    if (n == 0 || n >= (1ull << 28)) return dn_set_err(DN_CUDA_ERR_ARG, "map size %ux%ux%u", sx, sy, sz);
    DNgpuVolume* g = new (std::nothrow) DNgpuVolume();
    if (!g) return dn_set_err(DN_CUDA_ERR_NOMEM, "host allocation");
    memset(g, 0, sizeof(*g));
    g->device = g_device;
    g->numSMs = g_numSMs;
    g->sx = sx; g->sy = sy; g->sz = sz; g->ntiles = n;
    int rc = DN_CUDA_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete g; return dn_set_err(DN_CUDA_ERR_LAUNCH, "stream: %s", cudaGetErrorString(e)); }
    g->ownStream = g->stream;
    e = cudaEventCreateWithFlags(&g->stageFree[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->stageFree[1], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->copyDone, cudaEventDisableTiming);
    if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "event: %s", cudaGetErrorString(e));
    if (!rc) rc = alloc_tiles(g);
    if (!rc) rc = valloc(g, g->rec, slotCap);
    if (!rc) rc = valloc(g, g->nsamples, slotCap);
    if (!rc) rc = valloc(g, g->vox, voxelCap);
    if (!rc) rc = valloc(g, g->diff, voxelCap);
    if (!rc) rc = valloc(g, g->spec, voxelCap);
    if (!rc) rc = valloc(g, g->st, 1);
    if (!rc) rc = valloc(g, g->dtab, 1);
    if (!rc) rc = reserve_requests(g, 1024);
    if (!rc) {
        COUNT_ALLOC();
        e = cudaMallocHost((void**)&g->hst, sizeof(DevState));
        if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_NOMEM, "pinned: %s", cudaGetErrorString(e));
    }
    if (!rc) {
        e = cudaMemsetAsync(g->st, 0, sizeof(DevState), g->stream);
        if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
    }
    if (rc) { dn_cuda_map_destroy(g); return rc; }
    g->slotCap = slotCap ? slotCap : 1;
    g->voxCap = voxelCap ? voxelCap : 1;
    *out = g;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_map_resize(DNgpuVolume* g, uint32_t sx, uint32_t sy, uint32_t sz)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    uint64_t n = (uint64_t)sx * sy * sz;
    if (n == 0 || n >= (1ull << 28)) return dn_set_err(DN_CUDA_ERR_ARG, "map size %ux%ux%u", sx, sy, sz);
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    free_tiles(g);
    g->sx = sx; g->sy = sy; g->sz = sz; g->ntiles = n;
    // request words name tiles of the old size: drop the list
    CK(cudaMemsetAsync(&g->st->w[ST_REQ], 0, 4, g->stream));
    return alloc_tiles(g);
}

template <class T> static int grow_copy(DNgpuVolume* g, T** p, uint64_t oldCount, uint64_t newCount)
{
    T* np = nullptr;
    const uint32_t bit = vol_array_bit(g, p);
    COUNT_ALLOC();
    if (g_asyncAlloc && bit) CK(cudaMallocAsync((void**)&np, (newCount ? newCount : 1) * sizeof(T), g->stream));
    else CK(cudaMalloc((void**)&np, (newCount ? newCount : 1) * sizeof(T)));
    if (*p && oldCount) CK(cudaMemcpyAsync(np, *p, oldCount * sizeof(T), cudaMemcpyDeviceToDevice, g->stream));
    // an array from the stream-ordered pool is freed after the copy and after every earlier use on the
    // volume's stream (a batch member's stream is the batch's: the frames in flight that still read it come
    // first), so the host does not wait; the host reads of these arrays synchronise the stream first, and
    // eviction orders its copies after it by an event.  Only a plain cudaFree needs the wait.
    if (!(bit && (g->poolMask & bit))) CK(cudaStreamSynchronize(g->stream));
    vfree(g, *p);
    *p = np;
    if (g_asyncAlloc && bit) g->poolMask |= bit;
    dn_new_generation(g);
    return DN_CUDA_OK;
}

// ------------------------------------------------------------ eviction
//
// A map's persistent device state -- tile arrays, records and sample counts, the voxel pool with its FP32
// lighting, the request list and the status block -- is what DN_sync_gpu, DN_draw and DN_update_lighting
// read and write between frames.  Eviction moves exactly that to pinned host memory and frees every
// device array of the map (scratch included); restoring allocates and copies it back.  The map's results
// after a restore are the ones it would have had without the round trip.

struct PersistentArray { void** ptr; size_t bytes; };

static int persistent_arrays(DNgpuVolume* g, PersistentArray* out)
{
    const uint64_t n = g->ntiles;
    int k = 0;
    out[k++] = {(void**)&g->tword, n * 4};
    out[k++] = {(void**)&g->treq, n};
    out[k++] = {(void**)&g->tvis, n};
    out[k++] = {(void**)&g->ttouch, n};
    out[k++] = {(void**)&g->tbits, (n + 31) / 32 * 8};
    out[k++] = {(void**)&g->tlast, n * 4};
    out[k++] = {(void**)&g->tpend, n * 4};
    out[k++] = {(void**)&g->tpendSlot, n * 4};
    out[k++] = {(void**)&g->rec, (size_t)g->slotCap * sizeof(ChunkRec)};
    out[k++] = {(void**)&g->nsamples, (size_t)g->slotCap * 4};
    out[k++] = {(void**)&g->vox, (size_t)g->voxCap * 8};
    out[k++] = {(void**)&g->diff, (size_t)g->voxCap * 16};
    out[k++] = {(void**)&g->spec, (size_t)g->voxCap * 16};
    out[k++] = {(void**)&g->reqs, (size_t)g->reqCap * 4};
    out[k++] = {(void**)&g->st, sizeof(DevState)};
    out[k++] = {(void**)&g->dtab, sizeof(LightTables)};
    return k;
}


extern "C" uint64_t dn_cuda_map_footprint(DNgpuVolume* g)
{
    if (!g) return 0;
    PersistentArray a[16];
    const int k = persistent_arrays(g, a);
    uint64_t total = 0;
    for (int i = 0; i < k; i++) total += a[i].bytes;
    total += (uint64_t)g->reqCap * 64 * sizeof(float4) + g->dstageCap + (uint64_t)g->dimgCap * 21;
    return total;
}

extern "C" int dn_cuda_map_is_resident(DNgpuVolume* g) { return g && !g->evicted; }

// pins slabs until the pool holds 'bytes' (free or in use); returns false when pinning fails
static bool slabs_grow_to(size_t bytes)
{
    while (g_slabs.size() * HOST_SLAB < bytes) {
        HostSlab sl{nullptr, nullptr};
        COUNT_ALLOC();
        if (cudaMallocHost((void**)&sl.p, HOST_SLAB) != cudaSuccess) { cudaGetLastError(); return false; }
        if (cudaEventCreateWithFlags(&sl.lastRead, cudaEventDisableTiming) != cudaSuccess) {
            cudaFreeHost(sl.p);
            cudaGetLastError();
            return false;
        }
        g_freeSlabs.push_back((uint32_t)g_slabs.size());
        g_slabs.push_back(sl);
    }
    return true;
}

extern "C" int dn_cuda_host_reserve(uint64_t bytes)
{
    if (g_device < 0) return dn_set_err(DN_CUDA_ERR_DEVICE, "dn_cuda_init was not called");
    CK(cudaSetDevice(g_device));
    std::lock_guard<std::mutex> lock(g_slabMutex);
    if (!slabs_grow_to((size_t)bytes)) return dn_set_err(DN_CUDA_ERR_NOMEM, "pinning %llu bytes of host memory failed",
                                                         (unsigned long long)bytes);
    return DN_CUDA_OK;
}

extern "C" uint64_t dn_cuda_host_pinned(void)
{
    std::lock_guard<std::mutex> lock(g_slabMutex);
    return (uint64_t)g_slabs.size() * HOST_SLAB;
}

extern "C" uint64_t dn_cuda_host_slab_bytes(void) { return (uint64_t)HOST_SLAB; }

extern "C" uint64_t dn_cuda_host_pinned_free(void)
{
    std::lock_guard<std::mutex> lock(g_slabMutex);
    return (uint64_t)g_freeSlabs.size() * HOST_SLAB;
}

extern "C" int dn_cuda_host_headroom(uint64_t bytes)
{
    if (g_device < 0) return dn_set_err(DN_CUDA_ERR_DEVICE, "dn_cuda_init was not called");
    CK(cudaSetDevice(g_device));
    std::lock_guard<std::mutex> lock(g_slabMutex);
    const size_t want = (size_t)((bytes + HOST_SLAB - 1) / HOST_SLAB);
    if (g_freeSlabs.size() >= want) return DN_CUDA_OK;
    if (!slabs_grow_to((g_slabs.size() + want - g_freeSlabs.size()) * HOST_SLAB))
        return dn_set_err(DN_CUDA_ERR_NOMEM, "pinning %llu more bytes of host memory failed", (unsigned long long)bytes);
    return DN_CUDA_OK;
}

// the eviction (restore = false) or restore copy stream of the current device (created on first use)
static int copy_stream(cudaStream_t* out, bool restore)
{
    std::lock_guard<std::mutex> lock(g_slabMutex);
    if (!g_copyStream || g_copyStreamDevice != g_device) {
        CK(cudaStreamCreateWithFlags(&g_copyStream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&g_restoreStream, cudaStreamNonBlocking));
        g_copyStreamDevice = g_device;
    }
    *out = restore ? g_restoreStream : g_copyStream;
    return DN_CUDA_OK;
}

// Eviction and restore never wait for the device.  Eviction waits (on the device, on the eviction stream)
// for the work queued on the volume's stream (the batch's stream while the volume is a member), then queues
// the copies of the persistent arrays into slabs of the pinned pool and the stream-ordered frees of the
// arrays; restore waits (on the restore stream) for the volume's eviction, queues the allocations and the
// copies back, returns the slabs with an event after the copies, and makes the volume's stream wait for
// them.  The copies so run beside the kernels of other maps.  Only slabs the pool does not hold yet are
// pinned (dn_cuda_host_reserve pins them ahead).
extern "C" int dn_cuda_map_evict(DNgpuVolume* g)
{
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    if (g->evicted) return DN_CUDA_OK;
    CK(cudaSetDevice(g->device));
    map_evicted(g);   // a restore still copying: the volume's stream (and so this eviction) waits for it
    PersistentArray a[16];
    const int k = persistent_arrays(g, a);
    size_t total = 0;
    for (int i = 0; i < k; i++) total += a[i].bytes;
    const uint32_t n = (uint32_t)((total + HOST_SLAB - 1) / HOST_SLAB);
    cudaStream_t cs;
    int rc0 = copy_stream(&cs, false);
    if (rc0) return rc0;
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    if (!ids) return dn_set_err(DN_CUDA_ERR_NOMEM, "host");
    {
        std::lock_guard<std::mutex> lock(g_slabMutex);
        if (g_freeSlabs.size() < n && !slabs_grow_to((g_slabs.size() + n - g_freeSlabs.size()) * HOST_SLAB)) {
            free(ids);
            return dn_set_err(DN_CUDA_ERR_NOMEM, "evict: pinning host memory for %llu bytes failed", (unsigned long long)total);
        }
        for (uint32_t i = 0; i < n; i++) { ids[i] = g_freeSlabs.back(); g_freeSlabs.pop_back(); }
    }
    // the volume's queued work, and the slabs' last readers (earlier restores), finish first, on the device
    CK(cudaEventRecord(g->copyDone, g->stream));
    CK(cudaStreamWaitEvent(cs, g->copyDone, 0));
    for (uint32_t i = 0; i < n; i++) CK(cudaStreamWaitEvent(cs, g_slabs[ids[i]].lastRead, 0));
    // the arrays back to back across the slabs
    uint32_t si = 0;
    size_t so = 0;
    for (int i = 0; i < k; i++) {
        size_t done = 0;
        while (done < a[i].bytes) {
            const size_t len = (a[i].bytes - done) < (HOST_SLAB - so) ? (a[i].bytes - done) : (HOST_SLAB - so);
            cudaError_t e = cudaMemcpyAsync(g_slabs[ids[si]].p + so, (const unsigned char*)*a[i].ptr + done, len,
                                            cudaMemcpyDeviceToHost, cs);
            if (e != cudaSuccess) {
                cudaStreamSynchronize(cs);
                std::lock_guard<std::mutex> lock(g_slabMutex);
                for (uint32_t j = 0; j < n; j++) g_freeSlabs.push_back(ids[j]);
                free(ids);
                return dn_set_err(DN_CUDA_ERR_LAUNCH, "evict: %s", cudaGetErrorString(e));
            }
            done += len;
            so += len;
            if (so == HOST_SLAB) { so = 0; si++; }
        }
    }
    // the frees follow the copies in the copy stream's order; the arrays that are not copied (scratch) were
    // last used on the volume's stream, which the copy stream waited for
    free_tiles(g, cs);
    vfree(g, g->rec, cs); vfree(g, g->nsamples, cs); vfree(g, g->vox, cs); vfree(g, g->diff, cs); vfree(g, g->spec, cs);
    vfree(g, g->reqs, cs); vfree(g, g->st, cs); vfree(g, g->dtab, cs);
    vfree(g, g->lightOut, cs); vfree(g, g->dstage, cs); vfree(g, g->dimg, cs); vfree(g, g->dhit, cs); vfree(g, g->dface, cs);
    g->dstageCap = 0; g->dimgCap = 0;
    CK(cudaEventRecord(g->copyDone, cs));
    g->evicted = ids;
    g->evictedSlabs = n;
    dn_new_generation(g);
    return DN_CUDA_OK;
}

// the allocations and copies of a restore, on the restore stream; copyDone marks their end
static int restore_copies(DNgpuVolume* g);

extern "C" int dn_cuda_map_restore(DNgpuVolume* g)
{
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    if (!g->evicted) { map_evicted(g); return DN_CUDA_OK; }
    int rc = restore_copies(g);
    if (rc) return rc;
    // the volume's later work waits for its arrays
    CK(cudaStreamWaitEvent(g->stream, g->copyDone, 0));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_map_restore_async(DNgpuVolume* g)
{
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    if (!g->evicted) return DN_CUDA_OK;
    CK(cudaSetDevice(g->device));
    int rc = restore_copies(g);
    if (rc) return rc;
    g->restorePending = 1;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_map_restore_query(DNgpuVolume* g)
{
    if (!g) { dn_set_err(DN_CUDA_ERR_ARG, "null volume"); return -1; }
    if (g->evicted) return 0;
    if (!g->restorePending) return 1;
    CK(cudaSetDevice(g->device));
    const cudaError_t e = cudaEventQuery(g->copyDone);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    dn_set_err(DN_CUDA_ERR_LAUNCH, "restore: %s", cudaGetErrorString(e));
    return -1;
}

static int restore_copies(DNgpuVolume* g)
{
    PersistentArray a[16];
    const int k = persistent_arrays(g, a);
    cudaStream_t cs;
    int rc = copy_stream(&cs, true);
    if (rc) return rc;
    CK(cudaStreamWaitEvent(cs, g->copyDone, 0));   // the eviction's copies into the slabs, and its frees
    // the arrays in persistent_arrays' order, each from the pool on the restore stream
    rc = valloc(g, g->tword, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->treq, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->tvis, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->ttouch, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->tbits, (g->ntiles + 31) / 32 * 2, cs);
    if (!rc) rc = valloc(g, g->tlast, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->tpend, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->tpendSlot, g->ntiles, cs);
    if (!rc) rc = valloc(g, g->rec, g->slotCap, cs);
    if (!rc) rc = valloc(g, g->nsamples, g->slotCap, cs);
    if (!rc) rc = valloc(g, g->vox, g->voxCap, cs);
    if (!rc) rc = valloc(g, g->diff, g->voxCap, cs);
    if (!rc) rc = valloc(g, g->spec, g->voxCap, cs);
    if (!rc) rc = valloc(g, g->reqs, g->reqCap, cs);
    if (!rc) rc = valloc(g, g->st, 1, cs);
    if (!rc) rc = valloc(g, g->dtab, 1, cs);
    if (!rc) rc = valloc(g, g->lightOut, (size_t)g->reqCap * 64, cs);
    if (rc) {
        free_tiles(g, cs);
        vfree(g, g->rec, cs); vfree(g, g->nsamples, cs); vfree(g, g->vox, cs); vfree(g, g->diff, cs); vfree(g, g->spec, cs);
        vfree(g, g->reqs, cs); vfree(g, g->st, cs); vfree(g, g->dtab, cs); vfree(g, g->lightOut, cs);
        return rc;
    }
    uint32_t si = 0;
    size_t so = 0;
    for (int i = 0; i < k; i++) {
        size_t done = 0;
        while (done < a[i].bytes) {
            const size_t len = (a[i].bytes - done) < (HOST_SLAB - so) ? (a[i].bytes - done) : (HOST_SLAB - so);
            CK(cudaMemcpyAsync((unsigned char*)*a[i].ptr + done, g_slabs[g->evicted[si]].p + so, len,
                               cudaMemcpyHostToDevice, cs));
            done += len;
            so += len;
            if (so == HOST_SLAB) { so = 0; si++; }
        }
    }
    // the slabs are free for the next eviction once these copies have read them
    {
        std::lock_guard<std::mutex> lock(g_slabMutex);
        for (uint32_t i = 0; i < g->evictedSlabs; i++) {
            CK(cudaEventRecord(g_slabs[g->evicted[i]].lastRead, cs));
            g_freeSlabs.push_back(g->evicted[i]);
        }
    }
    CK(cudaEventRecord(g->copyDone, cs));
    free(g->evicted);
    g->evicted = nullptr;
    g->evictedSlabs = 0;
    dn_new_generation(g);
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_reserve(DNgpuVolume* g, uint32_t slotCap, uint64_t voxelCap, uint64_t requestCap)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    int rc;
    if (slotCap > g->slotCap) {
        if ((rc = grow_copy(g, &g->rec, g->slotCap, slotCap)) || (rc = grow_copy(g, &g->nsamples, g->slotCap, slotCap))) return rc;
        g->slotCap = slotCap;
    }
    if (voxelCap > g->voxCap) {
        if ((rc = grow_copy(g, &g->vox, g->voxCap, voxelCap)) || (rc = grow_copy(g, &g->diff, g->voxCap, voxelCap)) ||
            (rc = grow_copy(g, &g->spec, g->voxCap, voxelCap)))
            return rc;
        g->voxCap = voxelCap;
    }
    if (requestCap > g->reqCap && (rc = reserve_requests(g, requestCap))) return rc;
    return DN_CUDA_OK;
}

// ------------------------------------------------------------------ draw

__global__ void __launch_bounds__(256, DN_DRAW_MIN_BLOCKS) k_draw(const __grid_constant__ DrawArgs a)
{
    __shared__ Material smat[256];
    for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < 256; i += blockDim.x * blockDim.y) smat[i] = a.mats[i];
    __syncthreads();
    Counters c;
    const uint32_t primary = draw_pixel(a.d, smat, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y, c);
    flush_counters(a.d.stats, c, primary, 0);
}

// -------------------------------------------------------------- lighting

// The lighting launch as persistent per-lane ray streams (dn_light_stream.cuh).
__global__ void __launch_bounds__(128, DN_STREAM_MIN_BLOCKS) k_light_stream(const __grid_constant__ StreamArgs a)
{
    __shared__ StreamShared sh;
    // per-voxel job state lives in shared memory: it is touched only when a segment ends
    __shared__ Job jobs[128];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sh.mats[i] = a.mats[i];
    // shadow directions are identical for every voxel of the launch
    for (int k = threadIdx.x; k < 65; k += blockDim.x) shadow_dir(a.p, k, sh.sdir[k], sh.sinv[k]);
    __syncthreads();
    stream_loop<false>(&a, nullptr, &sh, jobs[threadIdx.x]);
}

// The lighting launch with specular and shadow fans traced as warp packets (dn_light_packet.cuh).
// the launch's materials and shadow directions into the volume's device tables, which k_light_packet
// reads through L1 (a kernel, not a copy from host memory, so that the launch sequence can be captured)
__global__ void k_light_tables(const __grid_constant__ MaterialTable t, const __grid_constant__ dn_light_params p,
                               LightTables* out)
{
    for (int i = threadIdx.x; i < 256; i += blockDim.x) out->mats[i] = t.m[i];
    for (int k = threadIdx.x; k < 65; k += blockDim.x) shadow_dir(p, k, out->sdir[k], out->sinv[k]);
}

__global__ void __launch_bounds__(128, DN_PACKET_MIN_BLOCKS) k_light_packet(const __grid_constant__ StreamArgs a)
{
    // shared memory holds only the four warps' pools (31 KB per block with 128-ray pools): 6 blocks fit
    // the 196 KB carveout, leaving about 60 KB of L1 for the map's masks and voxels; the tables are read
    // from a.gtab
    __shared__ PacketWarp warps[4];
    packet_loop<false>(&a, nullptr, warps[threadIdx.x >> 5]);
}

// the opaque-chunk marks of one map for a lighting launch with the given materials (mark_opaque_word)
__global__ void __launch_bounds__(256) k_mark_opaque(uint32_t* tbits, const uint32_t* tword, const ChunkRec* rec,
                                                     uint64_t nwords, const __grid_constant__ MaterialTable t)
{
    __shared__ uint32_t opq[8];
    opaque_materials(t.m, opq);
    for (uint64_t wi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; wi < nwords; wi += (uint64_t)gridDim.x * blockDim.x)
        mark_opaque_word(tbits, tword, rec, wi, opq);
}

// The diffuse paths of the voxels k_light_packet lit, as per-lane path streams over the whole request list:
// a lane whose voxel's paths are done takes the next voxel, so no lane waits for another lane's long path.
__global__ void __launch_bounds__(128, DN_DIFF_MIN_BLOCKS) k_light_diffuse(const __grid_constant__ StreamArgs a)
{
    __shared__ Job jobs[128];
    stream_loop<false, true>(&a, nullptr, nullptr, jobs[threadIdx.x]);
}

// launches the lighting kernel g_lightKernel selects (1 ray streams, 2 warp packets followed by the
// diffuse-path kernel; packets need specBounceLimit <= PK_MAX_SPEC_SEGMENTS and fall back to streams
// otherwise) with its batch threshold
static int launch_light(DNgpuVolume* g, StreamArgs& a)
{
    int perSM = 0;
    MaterialTable table;                // on the stack: a launch argument, copied at the launch
    memcpy(table.m, a.mats, sizeof(table.m));
    {
        const uint64_t nwords = (g->ntiles + 15) / 16;
        const uint64_t blocks = (nwords + 255) / 256;
        const uint32_t maxBlocks = (uint32_t)(g->numSMs > 0 ? g->numSMs * 4 : 512);
        COUNT_LAUNCH();
        k_mark_opaque<<<(uint32_t)(blocks < maxBlocks ? blocks : maxBlocks), 256, 0, g->stream>>>(
            g->tbits, g->tword, g->rec, nwords, table);
        CK(cudaGetLastError());
    }
    if (g_lightKernel == 2 && a.p.specBounceLimit <= PK_MAX_SPEC_SEGMENTS) {
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light_packet, 128, 0));
        if (perSM < 1) perSM = 1;
        a.batch = g_packetBatch;
        a.gtab = g->dtab;
        COUNT_LAUNCH();
        k_light_tables<<<1, 256, 0, g->stream>>>(table, a.p, g->dtab);
        COUNT_LAUNCH();
        k_light_packet<<<g->numSMs * perSM, 128, 0, g->stream>>>(a);
        CK(cudaGetLastError());
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light_diffuse, 128, 0));
        if (perSM < 1) perSM = 1;
        CK(cudaMemsetAsync(a.workCounter, 0, 4, g->stream));
        a.batch = g_streamBatch;
        COUNT_LAUNCH();
        k_light_diffuse<<<g->numSMs * perSM, 128, 0, g->stream>>>(a);
    } else {
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light_stream, 128, 0));
        if (perSM < 1) perSM = 1;
        a.batch = g_streamBatch;
        COUNT_LAUNCH();
        k_light_stream<<<g->numSMs * perSM, 128, 0, g->stream>>>(a);
    }
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

// D1/D2: commit the new lighting after the whole launch, then count the sample
__global__ void k_commit(DevMap m, const uint32_t* reqs, const uint32_t* nreqPtr, const float4* out,
                         float4* diff, float4* spec, uint32_t* nsamples)
{
    const uint32_t nreq = *nreqPtr;
    const uint64_t total = (uint64_t)nreq * 32u;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
        commit_lane(m, reqs, out, i, (uint32_t)(i >> 5), (uint32_t)(i & 31u), diff, spec, nsamples);
}

// ------------------------------------------------------------------ sync

// applies the host's per-tile ops and writes staged chunk records + voxels (one block per op)
__global__ void k_sync_stage(const dn_tile_op* ops, uint32_t nops, const dn_chunk_record* recs,
                             const uint64_t* voxOff, const uint32_t* words, uint32_t* tpend, uint32_t* tpendSlot,
                             ChunkRec* rec, uint32_t* nsamples, uint2* vox, float4* diff, float4* spec,
                             uint32_t slotCap, uint64_t voxCap, uint64_t ntiles, DevState* st)
{
    for (uint32_t o = blockIdx.x; o < nops; o += gridDim.x) {
        const dn_tile_op op = ops[o];
        if (op.tile >= ntiles) { if (threadIdx.x == 0) atomicOr(&st->w[ST_ERR], ERRF_TILE); continue; }
        const bool staged = (op.flags & DN_PEND_STAGED) != 0;
        const dn_chunk_record* srcp = staged ? &recs[op.recordIndex] : nullptr;
        const bool bad = staged && (op.slot >= slotCap || srcp->nvox > 512u || (uint64_t)srcp->voxBase + srcp->nvox > voxCap);
        if (threadIdx.x == 0) {
            // a record that does not fit is not published: the tile stays unloaded
            tpend[op.tile] = bad ? (op.flags & ~DN_PEND_STAGED) : op.flags;
            tpendSlot[op.tile] = bad ? DN_SLOT_NONE : op.slot;
            if (bad) atomicOr(&st->w[ST_ERR], ERRF_RECORD);
        }
        if (!staged || bad) continue;
        const dn_chunk_record& src = *srcp;
        ChunkRec* dst = &rec[op.slot];
        const uint32_t* s32 = (const uint32_t*)&src;
        uint32_t* d32 = (uint32_t*)dst;
        __shared__ uint32_t mats[8];
        if (threadIdx.x < 8) mats[threadIdx.x] = 0;
        __syncthreads();
        if (threadIdx.x < 24) d32[threadIdx.x] = s32[threadIdx.x];
        if (threadIdx.x == 0) nsamples[op.slot] = 0;
        const uint64_t off = voxOff[op.recordIndex];
        for (uint32_t i = threadIdx.x; i < src.nvox; i += blockDim.x) {
            const uint64_t d = (uint64_t)src.voxBase + i;
            const uint32_t nw = words[2 * (off + i)];
            vox[d] = make_uint2(nw, words[2 * (off + i) + 1]);
            diff[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            spec[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            atomicOr(&mats[(nw >> 24) >> 5], 1u << ((nw >> 24) & 31u));
        }
        __syncthreads();
        if (threadIdx.x < 8) dst->matSet[threadIdx.x] = mats[threadIdx.x];
        __syncthreads();
    }
}

// Packs and publishes staged chunks from the voxels of the CPU map (one 512-thread block per op); the
// packing of voxel.c:1397-1461 restated per voxel.  Thread i is voxel i = x + 8*(y + 8*z), which is bit i
// of the occupancy mask, so warp w's ballot is mask word w; the CPU array is stored [x][y][z].  A solid
// voxel is kept when one of its six face neighbours is outside the chunk or see-through (voxel.c:1391-1394).
// Kept voxels go to the record's pool range in mask order (their rank), with linear albedo.  The host
// counted the kept voxels to size the range; a record whose count differs is not published.
__global__ void __launch_bounds__(512) k_pack_stage(const dn_tile_op* ops, uint32_t nops, const dn_chunk_record* recs,
                                                    const uint2* raw, const dn_pack_params* pk, uint32_t* tpend,
                                                    uint32_t* tpendSlot, ChunkRec* rec, uint32_t* nsamples, uint2* vox,
                                                    float4* diff, float4* spec, uint32_t slotCap, uint64_t voxCap,
                                                    uint64_t ntiles, DevState* st)
{
    __shared__ uint8_t thru[512];
    __shared__ uint8_t lin[256];
    __shared__ uint32_t see[8], maskW[16], mats[8];
    const uint32_t i = threadIdx.x, lane = i & 31u, warp = i >> 5;
    const uint32_t x = i & 7u, y = (i >> 3) & 7u, z = i >> 6;
    const uint32_t r = (x << 6) | (y << 3) | z;
    if (i < 8) see[i] = pk->seeThrough[i];
    if (i < 256) lin[i] = pk->linear[i];
    for (uint32_t o = blockIdx.x; o < nops; o += gridDim.x) {
        const dn_tile_op op = ops[o];
        __syncthreads();   // the previous op's shared-memory reads are done (and the tables are written)
        if (op.tile >= ntiles) { if (i == 0) atomicOr(&st->w[ST_ERR], ERRF_TILE); continue; }
        if (!(op.flags & DN_PEND_STAGED)) {
            if (i == 0) { tpend[op.tile] = op.flags; tpendSlot[op.tile] = op.slot; }
            continue;
        }
        const dn_chunk_record* src = &recs[op.recordIndex];
        const uint2 v = raw[(size_t)op.recordIndex * 512u + r];
        const uint32_t m = v.x >> 24;
        thru[i] = (uint8_t)((see[m >> 5] >> (m & 31u)) & 1u);
        if (i < 8) mats[i] = 0;
        __syncthreads();
        const bool keep = m != 255u &&
            (x == 7u || thru[i + 1] || x == 0u || thru[i - 1] || y == 7u || thru[i + 8] || y == 0u || thru[i - 8] ||
             z == 7u || thru[i + 64] || z == 0u || thru[i - 64]);
        const uint32_t ball = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) maskW[warp] = ball;
        __syncthreads();
        uint32_t before = 0, total = 0;
        #pragma unroll
        for (uint32_t w = 0; w < 16; w++) {
            const uint32_t c = __popc(maskW[w]);
            before += w < warp ? c : 0u;
            total += c;
        }
        const uint32_t nvox = src->nvox, base = src->voxBase;
        const bool bad = op.slot >= slotCap || nvox != total || (uint64_t)base + total > voxCap;
        if (i == 0) {
            tpend[op.tile] = bad ? (op.flags & ~DN_PEND_STAGED) : op.flags;
            tpendSlot[op.tile] = bad ? DN_SLOT_NONE : op.slot;
            if (bad) atomicOr(&st->w[ST_ERR], ERRF_RECORD);
        }
        if (bad) continue;
        if (keep) {
            const uint64_t d = (uint64_t)base + before + __popc(ball & ((1u << lane) - 1u));
            const uint32_t a = v.y;
            vox[d] = make_uint2(v.x, ((uint32_t)lin[a >> 24] << 24) | ((uint32_t)lin[(a >> 16) & 0xFFu] << 16) |
                                     ((uint32_t)lin[(a >> 8) & 0xFFu] << 8));
            diff[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            spec[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            atomicOr(&mats[m >> 5], 1u << (m & 31u));
        }
        __syncthreads();
        ChunkRec* dst = &rec[op.slot];
        if (i < 16) dst->mask[i] = maskW[i];
        else if (i < 19) {
            uint32_t c = 0;
            for (uint32_t w = 0; w < 4u * (i - 15u); w++) c += __popc(maskW[w]);
            dst->partial[i - 16] = c;
        } else if (i == 19) dst->nvox = total;
        else if (i < 23) dst->pos[i - 20] = src->pos[i - 20];
        else if (i == 23) dst->voxBase = base;
        else if (i < 32) dst->matSet[i - 24] = mats[i - 24];
        else if (i == 32) nsamples[op.slot] = 0;
    }
}

// DN_sync_gpu's per-tile pass (compact_tiles) over every tile of one map
__global__ void __launch_bounds__(256) k_compact(const __grid_constant__ CompactArgs a)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < a.ntiles; base += stride) compact_tiles(a, base);
}

__global__ void k_clamp_requests(DevState* st, uint64_t cap)
{
    if (st->w[ST_REQ] > cap) st->w[ST_REQ] = (uint32_t)cap;
}

static int stage_reserve(DNgpuVolume* g, size_t total, unsigned char** host, int* which);

int dn_stage_ops(DNgpuVolume* g, const dn_tile_op* ops, uint32_t nops, const dn_chunk_record* records,
                 uint32_t nrecords, const uint32_t* voxelWords, uint64_t nvoxels)
{
    if (nops) {
        // one pinned upload: ops | records | voxel offsets | voxel words
        const size_t bOps = (size_t)nops * sizeof(dn_tile_op);
        const size_t bRec = (size_t)nrecords * sizeof(dn_chunk_record);
        const size_t bOff = (size_t)nrecords * sizeof(uint64_t);
        const size_t bVox = (size_t)nvoxels * 8u;
        const size_t oRec = (bOps + 15) & ~(size_t)15, oOff = (oRec + bRec + 15) & ~(size_t)15,
                     oVox = (oOff + bOff + 15) & ~(size_t)15, total = oVox + bVox;
        unsigned char* hs = nullptr;
        int which = 0;
        int rc = stage_reserve(g, total, &hs, &which);
        if (rc) return rc;
        memcpy(hs, ops, bOps);
        if (bRec) memcpy(hs + oRec, records, bRec);
        uint64_t* off = (uint64_t*)(hs + oOff);
        uint64_t acc = 0;
        for (uint32_t r = 0; r < nrecords; r++) { off[r] = acc; acc += records[r].nvox; }
        if (acc != nvoxels) return dn_set_err(DN_CUDA_ERR_ARG, "voxel word count %llu != %llu", (unsigned long long)acc, (unsigned long long)nvoxels);
        for (uint32_t o = 0; o < nops; o++)
            if ((ops[o].flags & DN_PEND_STAGED) && ops[o].recordIndex >= nrecords)
                return dn_set_err(DN_CUDA_ERR_ARG, "op %u references record %u of %u", o, ops[o].recordIndex, nrecords);
        if (bVox) memcpy(hs + oVox, voxelWords, bVox);
        CK(cudaMemcpyAsync(g->dstage, hs, total, cudaMemcpyHostToDevice, g->stream));
        CK(cudaEventRecord(g->stageFree[which], g->stream));
        COUNT_LAUNCH();
        k_sync_stage<<<nops < 65535u ? nops : 65535u, 128, 0, g->stream>>>(
            (const dn_tile_op*)g->dstage, nops, (const dn_chunk_record*)(g->dstage + oRec),
            (const uint64_t*)(g->dstage + oOff), (const uint32_t*)(g->dstage + oVox), g->tpend, g->tpendSlot,
            g->rec, g->nsamples, g->vox, g->diff, g->spec, g->slotCap, g->voxCap, g->ntiles, g->st);
        CK(cudaGetLastError());
    }
    return DN_CUDA_OK;
}

static const size_t STAGE_PART_DEFAULT = (size_t)16 << 20;
static const size_t CHUNK_VOXEL_BYTES = 512u * 8u;
static size_t g_stagePart = STAGE_PART_DEFAULT;

extern "C" size_t dn_cuda_stage_part_limit(size_t bytes)
{
    const size_t prev = g_stagePart;
    g_stagePart = bytes ? bytes : STAGE_PART_DEFAULT;
    return prev;
}

// the pinned upload buffer for the next upload, grown to 'total' bytes, and the device staging buffer
// grown likewise: the last buffer when its upload is done, else the other one (waiting only for its older
// upload, normally long done)
static int stage_reserve(DNgpuVolume* g, size_t total, unsigned char** host, int* which)
{
    int k = g->stageCur;
    const cudaError_t q = cudaEventQuery(g->stageFree[k]);
    if (q == cudaErrorNotReady) {
        k ^= 1;
        CK(cudaEventSynchronize(g->stageFree[k]));
    } else if (q != cudaSuccess) {
        CK(q);
    }
    if (total > g->hstageCap[k]) {
        if (g->hstage[k]) cudaFreeHost(g->hstage[k]);
        g->hstage[k] = nullptr;
        g->hstageCap[k] = 0;
        size_t nc = total + total / 2 + 4096;
        COUNT_ALLOC();
        CK(cudaMallocHost((void**)&g->hstage[k], nc));
        g->hstageCap[k] = nc;
    }
    g->stageCur = k;
    *host = g->hstage[k];
    *which = k;
    if (total > g->dstageCap) {
        if (!(g->poolMask & vol_array_bit(g, &g->dstage))) CK(cudaStreamSynchronize(g->stream));
        vfree(g, g->dstage);
        size_t nc = total + total / 2 + 4096;
        int rc = valloc(g, g->dstage, nc);
        if (rc) { g->dstageCap = 0; return rc; }
        g->dstageCap = nc;
    }
    return DN_CUDA_OK;
}

// Staging with packing on the device: params | ops | records | chunk voxels, in parts of at most
// g_stagePart bytes (or one op); each part's ops name its own records (recordIndex rebased to the part)
static int dn_stage_chunks(DNgpuVolume* g, const dn_pack_params* pk, const dn_tile_op* ops, uint32_t nops,
                           const dn_chunk_record* records, uint32_t nrecords, const void* const* chunkVoxels)
{
    for (uint32_t o = 0; o < nops; o++)
        if ((ops[o].flags & DN_PEND_STAGED) && ops[o].recordIndex >= nrecords)
            return dn_set_err(DN_CUDA_ERR_ARG, "op %u references record %u of %u", o, ops[o].recordIndex, nrecords);
    for (uint32_t r = 0; r < nrecords; r++)
        if (!chunkVoxels[r] || records[r].nvox > 512u)
            return dn_set_err(DN_CUDA_ERR_ARG, "record %u: %s", r, chunkVoxels[r] ? "more than 512 voxels" : "no voxels");
    const size_t perOp = sizeof(dn_tile_op) + sizeof(dn_chunk_record) + CHUNK_VOXEL_BYTES;
    const size_t oOps = (sizeof(dn_pack_params) + 15) & ~(size_t)15;
    uint32_t o0 = 0;
    while (o0 < nops) {
        // the part: ops o0 .. o1-1, at most g_stagePart bytes (at least one op)
        uint32_t o1 = o0, nrec = 0;
        size_t bytes = oOps + 64;
        while (o1 < nops) {
            const bool staged = (ops[o1].flags & DN_PEND_STAGED) != 0;
            const size_t add = staged ? perOp : sizeof(dn_tile_op);
            if (o1 > o0 && bytes + add > g_stagePart) break;
            bytes += add;
            nrec += staged;
            o1++;
        }
        const uint32_t n = o1 - o0;
        const size_t oRec = (oOps + (size_t)n * sizeof(dn_tile_op) + 15) & ~(size_t)15;
        const size_t oVox = (oRec + (size_t)nrec * sizeof(dn_chunk_record) + 15) & ~(size_t)15;
        const size_t total = oVox + (size_t)nrec * CHUNK_VOXEL_BYTES;
        unsigned char* hs = nullptr;
        int which = 0;
        int rc = stage_reserve(g, total, &hs, &which);
        if (rc) return rc;
        memcpy(hs, pk, sizeof(dn_pack_params));
        dn_tile_op* hops = (dn_tile_op*)(hs + oOps);
        dn_chunk_record* hrec = (dn_chunk_record*)(hs + oRec);
        unsigned char* hvox = hs + oVox;
        uint32_t k = 0;
        for (uint32_t j = 0; j < n; j++) {
            dn_tile_op op = ops[o0 + j];
            if (op.flags & DN_PEND_STAGED) {
                hrec[k] = records[op.recordIndex];
                memcpy(hvox + (size_t)k * CHUNK_VOXEL_BYTES, chunkVoxels[op.recordIndex], CHUNK_VOXEL_BYTES);
                op.recordIndex = k++;
            }
            hops[j] = op;
        }
        CK(cudaMemcpyAsync(g->dstage, hs, total, cudaMemcpyHostToDevice, g->stream));
        CK(cudaEventRecord(g->stageFree[which], g->stream));
        COUNT_LAUNCH();
        k_pack_stage<<<n < 65535u ? n : 65535u, 512, 0, g->stream>>>(
            (const dn_tile_op*)(g->dstage + oOps), n, (const dn_chunk_record*)(g->dstage + oRec),
            (const uint2*)(g->dstage + oVox), (const dn_pack_params*)g->dstage, g->tpend, g->tpendSlot, g->rec,
            g->nsamples, g->vox, g->diff, g->spec, g->slotCap, g->voxCap, g->ntiles, g->st);
        CK(cudaGetLastError());
        o0 = o1;
    }
    return DN_CUDA_OK;
}

// the per-tile pass of a sync after its staging (compact_tiles), then the request count's clamp
static int sync_tiles(DNgpuVolume* g, const dn_sync_params* p)
{
    CK(cudaMemsetAsync(&g->st->w[ST_REQ], 0, 4, g->stream));
    CompactArgs a;
    a.tword = g->tword; a.tbits = g->tbits; a.treq = g->treq; a.tvis = g->tvis; a.ttouch = g->ttouch; a.tlast = g->tlast;
    a.tpend = g->tpend; a.tpendSlot = g->tpendSlot; a.rec = g->rec;
    a.reqs = g->reqs; a.reqCap = g->reqCap; a.st = g->st; a.ntiles = g->ntiles;
    a.op = p->op; a.split = p->split; a.frameNum = p->frameNum;
    uint64_t blocks = (g->ntiles + 255) / 256;
    uint32_t maxBlocks = (uint32_t)(g->numSMs > 0 ? g->numSMs * 8 : 1024);
    COUNT_LAUNCH();
    k_compact<<<(uint32_t)(blocks < maxBlocks ? blocks : maxBlocks), 256, 0, g->stream>>>(a);
    CK(cudaGetLastError());
    COUNT_LAUNCH();
    k_clamp_requests<<<1, 1, 0, g->stream>>>(g->st, g->reqCap);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_sync_stage_chunks(DNgpuVolume* g, const dn_pack_params* pk, const dn_tile_op* ops, uint32_t nops,
                                         const dn_chunk_record* records, uint32_t nrecords, const void* const* chunkVoxels)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !pk || (nops && !ops) || (nrecords && (!records || !chunkVoxels))) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    CK(cudaSetDevice(g->device));
    return dn_stage_chunks(g, pk, ops, nops, records, nrecords, chunkVoxels);
}

extern "C" int dn_cuda_sync_chunks(DNgpuVolume* g, const dn_sync_params* p, const dn_pack_params* pk, const dn_tile_op* ops,
                                   uint32_t nops, const dn_chunk_record* records, uint32_t nrecords,
                                   const void* const* chunkVoxels)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !p || !pk || (nops && !ops) || (nrecords && (!records || !chunkVoxels))) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->split == 0 || p->op > 2) return dn_set_err(DN_CUDA_ERR_ARG, "bad sync parameters");
    CK(cudaSetDevice(g->device));
    int rc = dn_stage_chunks(g, pk, ops, nops, records, nrecords, chunkVoxels);
    if (rc) return rc;
    return sync_tiles(g, p);
}

extern "C" int dn_cuda_export_chunk(DNgpuVolume* g, uint32_t tile, dn_chunk_record* recOut, uint32_t matSet[8],
                                    uint32_t* words)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !recOut) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (tile >= g->ntiles) return dn_set_err(DN_CUDA_ERR_ARG, "tile %u of %llu", tile, (unsigned long long)g->ntiles);
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    uint32_t w = 0;
    CK(cudaMemcpy(&w, &g->tword[tile], 4, cudaMemcpyDeviceToHost));
    const uint32_t slot = w & dn::SLOT_MASK;
    if (slot == DN_SLOT_NONE || slot >= g->slotCap) return dn_set_err(DN_CUDA_ERR_ARG, "tile %u has no record", tile);
    ChunkRec r;
    CK(cudaMemcpy(&r, &g->rec[slot], sizeof(ChunkRec), cudaMemcpyDeviceToHost));
    if (r.nvox > 512u || (uint64_t)r.voxBase + r.nvox > g->voxCap)
        return dn_set_err(DN_CUDA_ERR_ARG, "tile %u: record out of range", tile);
    memcpy(recOut->mask, r.mask, sizeof(r.mask));
    memcpy(recOut->partial, r.partial, sizeof(r.partial));
    recOut->nvox = r.nvox;
    memcpy(recOut->pos, r.pos, sizeof(r.pos));
    recOut->voxBase = r.voxBase;
    if (matSet) memcpy(matSet, r.matSet, sizeof(r.matSet));
    if (words && r.nvox) CK(cudaMemcpy(words, &g->vox[r.voxBase], (size_t)r.nvox * 8u, cudaMemcpyDeviceToHost));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_sync_stage(DNgpuVolume* g, const dn_tile_op* ops, uint32_t nops, const dn_chunk_record* records,
                                  uint32_t nrecords, const uint32_t* voxelWords, uint64_t nvoxels)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    CK(cudaSetDevice(g->device));
    return dn_stage_ops(g, ops, nops, records, nrecords, voxelWords, nvoxels);
}

extern "C" int dn_cuda_sync(DNgpuVolume* g, const dn_sync_params* p, const dn_tile_op* ops, uint32_t nops,
                            const dn_chunk_record* records, uint32_t nrecords, const uint32_t* voxelWords,
                            uint64_t nvoxels)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !p) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->split == 0 || p->op > 2) return dn_set_err(DN_CUDA_ERR_ARG, "bad sync parameters");
    CK(cudaSetDevice(g->device));
    int rc = dn_stage_ops(g, ops, nops, records, nrecords, voxelWords, nvoxels);
    if (rc) return rc;
    return sync_tiles(g, p);
}

extern "C" int dn_cuda_light(DNgpuVolume* g, const dn_light_params* p, const dn_material* materials)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !p || !materials) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->K < 1 || p->K > 64) return dn_set_err(DN_CUDA_ERR_ARG, "K = %u", p->K);
    CK(cudaSetDevice(g->device));
    CK(cudaMemsetAsync(&g->st->w[ST_WORK], 0, 4, g->stream));
    static thread_local StreamArgs* a = nullptr;
    if (!a) a = new StreamArgs();
    a->m = dev_map(g);
    a->m.degen = &g->st->lstats[S_DEGEN];
    a->reqs = g->reqs; a->workCounter = &g->st->w[ST_WORK]; a->nreqPtr = &g->st->w[ST_REQ];
    a->nsamples = g->nsamples; a->out = g->lightOut; a->stats = g->st->lstats;
    a->batch = g_streamBatch;
    a->p = *p;
    memcpy(a->mats, materials, sizeof(a->mats));
    int rc = launch_light(g, *a);
    if (rc) return rc;
    COUNT_LAUNCH();
    k_commit<<<g->numSMs * 4, 256, 0, g->stream>>>(dev_map(g), g->reqs, &g->st->w[ST_REQ], g->lightOut, g->diff, g->spec,
                                                  g->nsamples);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

// ------------------------------------------------- lighting without allocation
//
// The lighting update keeps the new lighting of every request lane in scratch memory until the commit
// kernel copies it into the voxel pool.  dn_cuda_light uses the volume's own scratch, which
// dn_cuda_sync grows with cudaMalloc as the map's lit set grows.  Some callers cannot allow that:
// a render loop that runs under a fixed device-memory budget, or a host engine that hands out all
// device memory through its own allocator and forbids ad-hoc cudaMalloc / cudaFree while a frame is
// in flight.  dn_cuda_light_noalloc serves them: its scratch is the fixed array below, part of this
// library's device image (every GPU that loads the library holds it until the process exits), so the
// call itself allocates nothing on the device or the host.
//
// Limit: DN_NOALLOC_MAX_REQUESTS request groups (32 voxels each) per call.  The request count exists
// only on the device (the sync built it there), so the limit is checked there: k_noalloc_guard copies
// the count into ST_LIMITED, or 0 with the ERRF_NOALLOC_CAPACITY flag when it exceeds the limit; the
// lighting and commit kernels of the call light ST_LIMITED groups, so an oversized list is lit not at
// all and changes nothing, and the next dn_cuda_finish reports DN_CUDA_ERR_CAPACITY.  The host never
// waits for the device in this call.
// The array's device address is looked up once per device, on that device's first call (with the
// device current); that first call should come before any stream capture.  dn_cuda_init and
// dn_cuda_shutdown forget the looked-up addresses (a device reset invalidates them).  Every call
// shares the array and it keeps the previous call's contents: nothing in it needs to start at zero,
// because each call writes every slot it later reads.  Calls that overlap on the GPU (two volumes lit
// concurrently on different streams) race on the array.
#define DN_NOALLOC_MAX_REQUESTS 8192u   // 8192 groups x 32 lanes x 2 float4 = 8 MiB
static __device__ __align__(256) float4 g_noallocScratch[DN_NOALLOC_MAX_REQUESTS * 32u * 2u];
static_assert(sizeof(g_noallocScratch) == (size_t)DN_NOALLOC_MAX_REQUESTS * 32u * 2u * sizeof(float4),
              "one diffuse and one specular float4 per lane of every request group the limit admits");

static std::mutex g_noallocMutex;
static float4* g_noallocAddr[64];      // device address of g_noallocScratch, per device ordinal
static uint32_t g_noallocLimit = DN_NOALLOC_MAX_REQUESTS;

static void noalloc_forget(void)
{
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    memset(g_noallocAddr, 0, sizeof(g_noallocAddr));
}

static int noalloc_scratch(int device, float4** out)
{
    if (device < 0 || device >= 64) return dn_set_err(DN_CUDA_ERR_DEVICE, "device ordinal %d out of range", device);
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocAddr[device]) {
        float4* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noallocScratch);   // the device is current
        if (e != cudaSuccess || !ptr)
            return dn_set_err(DN_CUDA_ERR_LAUNCH, "cudaGetSymbolAddress of the fixed lighting scratch: %s", cudaGetErrorString(e));
        g_noallocAddr[device] = ptr;
    }
    *out = g_noallocAddr[device];
    return DN_CUDA_OK;
}

// the call's request count, or 0 and the capacity flag when the list exceeds the limit; the work counter
// of the lighting launch starts at zero
__global__ void k_noalloc_guard(DevState* st, uint32_t limit)
{
    const uint32_t n = st->w[ST_REQ];
    st->w[ST_LIMITED] = n <= limit ? n : 0u;
    if (n > limit) atomicOr(&st->w[ST_ERR], ERRF_NOALLOC_CAPACITY);
    st->w[ST_WORK] = 0;
}

extern "C" uint32_t dn_cuda_light_noalloc_set_limit(uint32_t groups)
{
    const uint32_t old = __atomic_load_n(&g_noallocLimit, __ATOMIC_RELAXED);
    const uint32_t v = (groups == 0u || groups > DN_NOALLOC_MAX_REQUESTS) ? DN_NOALLOC_MAX_REQUESTS : groups;
    __atomic_store_n(&g_noallocLimit, v, __ATOMIC_RELAXED);
    return old;
}

extern "C" int dn_cuda_light_noalloc(DNgpuVolume* g, const dn_light_params* p, const dn_material* materials)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !p || !materials) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->K < 1 || p->K > 64) return dn_set_err(DN_CUDA_ERR_ARG, "K = %u", p->K);
    CK(cudaSetDevice(g->device));
    float4* scratch = nullptr;
    int rc = noalloc_scratch(g->device, &scratch);
    if (rc) return rc;
    COUNT_LAUNCH();
    k_noalloc_guard<<<1, 1, 0, g->stream>>>(g->st, __atomic_load_n(&g_noallocLimit, __ATOMIC_RELAXED));
    CK(cudaGetLastError());
    StreamArgs a;                       // launch arguments on the stack: no host allocation either
    a.m = dev_map(g);
    a.m.degen = &g->st->lstats[S_DEGEN];
    a.reqs = g->reqs; a.workCounter = &g->st->w[ST_WORK]; a.nreqPtr = &g->st->w[ST_LIMITED];
    a.nsamples = g->nsamples; a.out = scratch; a.stats = g->st->lstats;
    a.batch = g_streamBatch;
    a.p = *p;
    memcpy(a.mats, materials, sizeof(a.mats));
    rc = launch_light(g, a);
    if (rc) return rc;
    COUNT_LAUNCH();
    k_commit<<<g->numSMs * 4, 256, 0, g->stream>>>(dev_map(g), g->reqs, &g->st->w[ST_LIMITED], scratch, g->diff, g->spec,
                                                  g->nsamples);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

int dn_reserve_image_staging(DNgpuVolume* g, size_t n)
{
    if (n <= g->dimgCap) return DN_CUDA_OK;
    CK(cudaStreamSynchronize(g->stream));
    vfree(g, g->dimg); vfree(g, g->dhit); vfree(g, g->dface);
    dn_new_generation(g);
    int rc;
    if ((rc = valloc(g, g->dimg, n)) || (rc = valloc(g, g->dhit, n)) || (rc = valloc(g, g->dface, n))) { g->dimgCap = 0; return rc; }
    g->dimgCap = n;
    return DN_CUDA_OK;
}

// The raster inputs of a draw: compose 0, or compose 1 with two buffers of device memory and non-zero
// sizes.  Checked before any launch, so that a bad pointer is an argument error, not a device fault.
int dn_check_raster(const dn_draw_params* p)
{
    if (p->compose == 0u) return DN_CUDA_OK;
    if (p->compose != 1u || !p->rasterColor || !p->rasterDepth || !p->rasterColorW || !p->rasterColorH ||
        !p->rasterDepthW || !p->rasterDepthH)
        return dn_set_err(DN_CUDA_ERR_ARG, "draw: invalid raster composition arguments (compose %u)", p->compose);
    const void* ptrs[2] = {p->rasterColor, p->rasterDepth};
    for (const void* q : ptrs) {
        cudaPointerAttributes at;
        const cudaError_t e = cudaPointerGetAttributes(&at, q);
        if (e != cudaSuccess || (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            (void)cudaGetLastError();
            return dn_set_err(DN_CUDA_ERR_ARG, "draw: raster texture %p is not device memory", q);
        }
    }
    return DN_CUDA_OK;
}

static int launch_draw(DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials, float4* color,
                       uint32_t* hit, uint8_t* face)
{
    const int rc = dn_check_raster(p);
    if (rc) return rc;
    static thread_local DrawArgs* a = nullptr;
    if (!a) a = new DrawArgs();
    a->d.m = dev_map(g);
    a->d.m.degen = &g->st->stats[S_DEGEN];
    a->d.p = *p;
    a->d.color = color; a->d.hit = hit; a->d.face = face; a->d.stats = g->st->stats;
    memcpy(a->mats, materials, sizeof(a->mats));
#ifndef DN_DRAW_BX
// 8 x 32 pixels per block: 16 x 16 and 32 x 8 measured equal or slower (large map: draw + sync 0.78 ms
// per frame with 8 x 32, 0.81 with 16 x 16, 0.89 with 32 x 8)
#define DN_DRAW_BX 8
#define DN_DRAW_BY 32
#endif
    dim3 block(DN_DRAW_BX, DN_DRAW_BY);
    dim3 grid((p->width + DN_DRAW_BX - 1) / DN_DRAW_BX, (p->height + DN_DRAW_BY - 1) / DN_DRAW_BY);
    COUNT_LAUNCH();
    k_draw<<<grid, block, 0, g->stream>>>(*a);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_draw(DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials, float* colorOut,
                            uint32_t* hitOut, uint8_t* faceOut)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !p || !materials || !colorOut) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->width == 0 || p->height == 0) return dn_set_err(DN_CUDA_ERR_ARG, "empty image");
    CK(cudaSetDevice(g->device));
    return launch_draw(g, p, materials, (float4*)colorOut, hitOut, faceOut);
}

extern "C" int dn_cuda_draw_host(DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials,
                                 float* colorOut, uint32_t* hitOut, uint8_t* faceOut)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !p || !materials || !colorOut) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->width == 0 || p->height == 0) return dn_set_err(DN_CUDA_ERR_ARG, "empty image");
    CK(cudaSetDevice(g->device));
    const size_t n = (size_t)p->width * p->height;
    int rc = dn_reserve_image_staging(g, n);
    if (rc) return rc;
    rc = launch_draw(g, p, materials, g->dimg, hitOut ? g->dhit : nullptr, faceOut ? g->dface : nullptr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(colorOut, g->dimg, n * 16, cudaMemcpyDeviceToHost, g->stream));
    if (hitOut) CK(cudaMemcpyAsync(hitOut, g->dhit, n * 4, cudaMemcpyDeviceToHost, g->stream));
    if (faceOut) CK(cudaMemcpyAsync(faceOut, g->dface, n, cudaMemcpyDeviceToHost, g->stream));
    return DN_CUDA_OK;
}

// ----------------------------------------------------------- introspection

extern "C" int dn_cuda_finish(DNgpuVolume* g, uint64_t* numRequests)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    CK(cudaMemcpyAsync(g->hst, g->st, sizeof(DevState), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    if (numRequests) *numRequests = g->hst->w[ST_REQ];
    if (g->hst->w[ST_ERR]) {
        uint32_t e = g->hst->w[ST_ERR];
        cudaMemsetAsync(&g->st->w[ST_ERR], 0, 4, g->stream);
        if (e == ERRF_NOALLOC_CAPACITY)
            return dn_set_err(DN_CUDA_ERR_CAPACITY,
                              "dn_cuda_light_noalloc: the request list exceeded the fixed scratch of %u groups (%u voxels); "
                              "that lighting update was skipped; use dn_cuda_light for this map",
                              __atomic_load_n(&g_noallocLimit, __ATOMIC_RELAXED),
                              __atomic_load_n(&g_noallocLimit, __ATOMIC_RELAXED) * 32u);
        return dn_set_err(DN_CUDA_ERR_KERNEL, "kernel error flags 0x%x", e);
    }
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_stats_kind(DNgpuVolume* g, int kind, dn_stats* out)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !out || kind < 0 || kind > 2) return dn_set_err(DN_CUDA_ERR_ARG, "bad argument");
    int rc = dn_cuda_finish(g, nullptr);
    if (rc && rc != DN_CUDA_ERR_KERNEL) return rc;
    unsigned long long s[8];
    for (int k = 0; k < 8; k++)
        s[k] = (kind != 2 ? g->hst->stats[k] : 0ull) + (kind != 1 ? g->hst->lstats[k] : 0ull);
    out->rays = s[S_RAYS]; out->primary = s[S_PRIMARY]; out->outerSteps = s[S_OUTER];
    out->chunksEntered = s[S_ENTERED]; out->innerSteps = s[S_INNER]; out->hits = s[S_HITS]; out->litVoxels = s[S_LIT];
    out->degenerate = s[S_DEGEN];
    return rc;
}

extern "C" int dn_cuda_stats(DNgpuVolume* g, dn_stats* out) { return dn_cuda_stats_kind(g, 0, out); }

extern "C" int dn_cuda_reset_stats(DNgpuVolume* g)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    CK(cudaMemsetAsync(g->st->stats, 0, sizeof(g->st->stats) + sizeof(g->st->lstats), g->stream));
    return DN_CUDA_OK;
}

extern "C" void* dn_cuda_stream(DNgpuVolume* g) { return g ? (void*)g->stream : nullptr; }

extern "C" int dn_cuda_read_tile_flags(DNgpuVolume* g, uint8_t* requested, uint8_t* touched)
{
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    if (map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    CK(cudaSetDevice(g->device));
    CK(cudaMemcpyAsync(requested, g->treq, g->ntiles, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemcpyAsync(touched, g->ttouch, g->ntiles, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_export_tiles(DNgpuVolume* g, uint8_t* state, uint8_t* vis, uint32_t* lastUsed, uint32_t* samples)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g) return dn_set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    const uint64_t n = g->ntiles;
    uint32_t* tw = (uint32_t*)malloc(n * 4);
    uint8_t* rq = (uint8_t*)malloc(n);
    uint32_t* ns = (uint32_t*)malloc((size_t)g->slotCap * 4);
    if (!tw || !rq || !ns) { free(tw); free(rq); free(ns); return dn_set_err(DN_CUDA_ERR_NOMEM, "host"); }
    cudaError_t e = cudaMemcpy(tw, g->tword, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rq, g->treq, n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && samples) e = cudaMemcpy(ns, g->nsamples, (size_t)g->slotCap * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && vis) e = cudaMemcpy(vis, g->tvis, n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && lastUsed) e = cudaMemcpy(lastUsed, g->tlast, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(tw); free(rq); free(ns); return dn_set_err(DN_CUDA_ERR_LAUNCH, "copy: %s", cudaGetErrorString(e)); }
    for (uint64_t t = 0; t < n; t++) {
        uint32_t st = tw[t] >> 30;
        if (state) state[t] = (uint8_t)((st == 1u && rq[t]) ? 3u : st);
        if (samples) samples[t] = (st == 2u) ? ns[tw[t] & SLOT_MASK] : 0u;
    }
    free(tw); free(rq); free(ns);
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_export_requests(DNgpuVolume* g, uint32_t* out, uint64_t capacity, uint64_t* count)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !count) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    uint64_t n = 0;
    int rc = dn_cuda_finish(g, &n);
    if (rc) return rc;
    *count = n;
    if (out && n) CK(cudaMemcpy(out, g->reqs, (n < capacity ? n : capacity) * 4, cudaMemcpyDeviceToHost));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_export_lighting(DNgpuVolume* g, uint32_t* index, float* diff, float* spec, uint64_t capacity,
                                       uint64_t* count)
{
    if (g && map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "the map is evicted; restore it first");
    if (!g || !count) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    const uint64_t n = g->ntiles;
    uint32_t* tw = (uint32_t*)malloc(n * 4);
    ChunkRec* rec = (ChunkRec*)malloc((size_t)g->slotCap * sizeof(ChunkRec));
    if (!tw || !rec) { free(tw); free(rec); return dn_set_err(DN_CUDA_ERR_NOMEM, "host"); }
    cudaError_t e = cudaMemcpy(tw, g->tword, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rec, g->rec, (size_t)g->slotCap * sizeof(ChunkRec), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(tw); free(rec); return dn_set_err(DN_CUDA_ERR_LAUNCH, "copy: %s", cudaGetErrorString(e)); }
    uint64_t rows = 0;
    for (uint64_t t = 0; t < n; t++)
        if ((tw[t] >> 30) == 2u) rows += rec[tw[t] & SLOT_MASK].nvox;
    *count = rows;
    if (!index || !diff || !spec) { free(tw); free(rec); return DN_CUDA_OK; }
    float4* hd = (float4*)malloc((size_t)g->voxCap * 16);
    float4* hs = (float4*)malloc((size_t)g->voxCap * 16);
    if (!hd || !hs) { free(tw); free(rec); free(hd); free(hs); return dn_set_err(DN_CUDA_ERR_NOMEM, "host"); }
    e = cudaMemcpy(hd, g->diff, (size_t)g->voxCap * 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hs, g->spec, (size_t)g->voxCap * 16, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(tw); free(rec); free(hd); free(hs); return dn_set_err(DN_CUDA_ERR_LAUNCH, "copy: %s", cudaGetErrorString(e)); }
    uint64_t k = 0;
    const uint32_t VX = g->sx * 8u, VY = g->sy * 8u;
    for (uint64_t t = 0; t < n && k < capacity; t++) {
        if ((tw[t] >> 30) != 2u) continue;
        const ChunkRec& r = rec[tw[t] & SLOT_MASK];
        const uint32_t tx = (uint32_t)(t % g->sx), ty = (uint32_t)((t / g->sx) % g->sy), tz = (uint32_t)(t / ((uint64_t)g->sx * g->sy));
        uint32_t rank = 0;
        for (uint32_t li = 0; li < 512 && k < capacity; li++) {
            if (!((r.mask[li >> 5] >> (li & 31)) & 1u)) continue;
            const uint32_t gx = tx * 8u + (li & 7u), gy = ty * 8u + ((li >> 3) & 7u), gz = tz * 8u + (li >> 6);
            index[k] = gx + VX * (gy + VY * gz);
            const float4 d = hd[r.voxBase + rank], s = hs[r.voxBase + rank];
            diff[3 * k] = d.x; diff[3 * k + 1] = d.y; diff[3 * k + 2] = d.z;
            spec[3 * k] = s.x; spec[3 * k + 1] = s.y; spec[3 * k + 2] = s.z;
            rank++; k++;
        }
    }
    free(tw); free(rec); free(hd); free(hs);
    return DN_CUDA_OK;
}

// ---------------------------------------------------------------- helpers

extern "C" int dn_cuda_malloc(void** p, size_t bytes) { COUNT_ALLOC(); CK(cudaMalloc(p, bytes ? bytes : 1)); return DN_CUDA_OK; }
extern "C" int dn_cuda_free(void* p) { if (p) CK(cudaFree(p)); return DN_CUDA_OK; }
extern "C" int dn_cuda_malloc_host(void** p, size_t bytes) { COUNT_ALLOC(); CK(cudaMallocHost(p, bytes ? bytes : 1)); return DN_CUDA_OK; }
extern "C" int dn_cuda_free_host(void* p) { if (p) CK(cudaFreeHost(p)); return DN_CUDA_OK; }
extern "C" int dn_cuda_memcpy_d2h(void* dst, const void* src, size_t bytes) { CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost)); return DN_CUDA_OK; }
// cudaMemcpy from pageable memory may return before the DMA has landed; the legacy-stream synchronise makes
// the bytes visible to work issued afterwards on the library's non-blocking streams
extern "C" int dn_cuda_memcpy_h2d(void* dst, const void* src, size_t bytes)
{
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(cudaStreamLegacy));
    return DN_CUDA_OK;
}
extern "C" int dn_cuda_event_create(void** ev) { CK(cudaEventCreate((cudaEvent_t*)ev)); return DN_CUDA_OK; }
extern "C" int dn_cuda_event_destroy(void* ev) { CK(cudaEventDestroy((cudaEvent_t)ev)); return DN_CUDA_OK; }
extern "C" int dn_cuda_event_record(void* ev, void* stream) { CK(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream)); return DN_CUDA_OK; }
extern "C" int dn_cuda_event_query(void* ev)
{
    cudaError_t e = cudaEventQuery((cudaEvent_t)ev);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    dn_set_err(DN_CUDA_ERR_LAUNCH, "event query: %s", cudaGetErrorString(e));
    return -1;
}
extern "C" int dn_cuda_event_elapsed_ms(void* s, void* e, float* ms) { CK(cudaEventElapsedTime(ms, (cudaEvent_t)s, (cudaEvent_t)e)); return DN_CUDA_OK; }
extern "C" int dn_cuda_stream_sync(void* stream) { CK(cudaStreamSynchronize((cudaStream_t)stream)); return DN_CUDA_OK; }
extern "C" int dn_cuda_device_sync(void) { CK(cudaDeviceSynchronize()); return DN_CUDA_OK; }

__global__ void k_flush(uint4* buf, size_t n, uint32_t v)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = make_uint4(v, v + 1, v + 2, v + 3);
}

extern "C" int dn_cuda_flush_l2(void* stream, size_t bytes)
{
    static uint4* buf = nullptr;
    static size_t cap = 0;
    static uint32_t tick = 0;
    size_t n = bytes / 16;
    if (n > cap) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        COUNT_ALLOC();
        CK(cudaMalloc((void**)&buf, n * 16));
        cap = n;
    }
    COUNT_LAUNCH();
    k_flush<<<g_numSMs > 0 ? g_numSMs * 4 : 256, 256, 0, (cudaStream_t)stream>>>(buf, n, tick++);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

extern "C" const char* dn_cuda_kernel_names(void)
{
    return "k_draw;k_light_stream;k_light_packet;k_light_diffuse;k_light_tables;k_mark_opaque;k_commit;k_sync_stage;k_pack_stage;k_compact;k_clamp_requests;k_flush;"
           "k_draw_batch;k_compact_batch;k_batch_reset;k_batch_prep;k_mark_opaque_batch;k_light_stream_batch;k_light_packet_batch;"
           "k_light_diffuse_batch;k_commit_batch;k_batch_gather;"
           "k_shape_count;k_shape_write";
}
