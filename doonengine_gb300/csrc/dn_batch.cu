/*
 * dn_batch.cu -- batched frames over many maps (the dn_cuda_batch_* entries of include/dn_cuda.h).
 *
 * A frame of a batch is a fixed handful of device operations whatever the number of maps:
 *   1. one host-to-device copy of the frame's table (per-map parameters, image pointers, materials);
 *   2. k_batch_reset: zero the request counters of the maps whose per-tile pass runs;
 *   3. k_draw_batch: every pixel of every image (blocks of 8x32 pixels; a block belongs to one map);
 *   4. k_compact_batch: the per-tile sync pass over every tile of every map (blocks of 256 tiles);
 *   5. k_batch_prep: clamp the request counts, lay the maps' request lists end to end as one queue (an
 *      exclusive prefix over the counts) and compute each map's shadow directions;
 *   6. k_light_stream_batch: the persistent lighting loop (dn_light_stream.cuh) over the whole queue;
 *   7. k_commit_batch: commit every map's new lighting.
 * Host-memory images are copied back on a second stream that overlaps steps 4-7.  A frame whose
 * composition repeats is captured once and replayed as a CUDA graph.
 *
 * Each map's results equal those of its single-map calls: the kernels run the same per-pixel, per-tile
 * and per-voxel code as dn_cuda.cu, every map's work reads and writes only that map's arrays, and the
 * lighting of a voxel does not depend on which lane, warp or launch computes it.
 */
#include "dn_internal.cuh"
#include "dn_light_stream.cuh"
#include "dn_light_packet.cuh"
#include <string.h>
#include <stddef.h>
#include <new>
#include <vector>
#include <algorithm>

using namespace dn;

struct BatchDrawEntry {
    DrawMap d;
    const Material* mats;
    uint32_t gridX;             // blocks of 8 pixels across
};

struct DNgpuBatch {
    int device;
    cudaStream_t stream, side;
    cudaEvent_t drawDone, copiesDone, tableFree;
    std::vector<DNgpuVolume*> members;
    unsigned char* htab; unsigned char* dtab; size_t tabCap;
    uint64_t tabGen;
    uint32_t* workCounter;
    DevState* bst;              // counters of batched launches (device)
    DevState* hbst;             // pinned copy
    unsigned long long* lsave;  // lighting counters saved around autotuning (device)
    DevState** dsts; uint32_t dstsCap; bool stsDirty;
    uint32_t* dgather; uint32_t* hgather;
    std::vector<DevState*> gatherHost;  // the pointer list last copied to dsts
    uint32_t gatherCount;
    dn_batch_tuning tuning;
    int maxBlocksPerSM;         // of the ray-stream kernel
    int maxBlocksPacket;        // of the packet kernel with PK_POOL_FAN-ray pools
    int maxBlocksPacketAlt;     // of the packet kernel with the other pool size (PK_POOL_ALT)
    int maxBlocksDiffuse;       // of the diffuse-path kernel that follows it
    std::vector<uint64_t> lastKey;
    std::vector<uint64_t> graphKey;
    cudaGraphExec_t graph;
    // the lighting launch of the last frame (autotuning re-runs it) and the generations of its maps
    BatchLightArgs lastLight;
    bool lastLightValid;
    bool lastPackets;
    std::vector<std::pair<DNgpuVolume*, uint64_t>> lastLightGens;
};

// ------------------------------------------------------------------ kernels

// largest i < n with start[i] <= v (start[0] = 0, non-decreasing): the entry whose range holds v
__device__ __forceinline__ uint32_t find_range(const uint32_t* start, uint32_t n, uint32_t v)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&start[mid]) <= v) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void k_batch_reset(const CompactArgs* s, uint32_t ns)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ns) s[i].st->w[ST_REQ] = 0;
}

__global__ void __launch_bounds__(256, DN_DRAW_MIN_BLOCKS) k_draw_batch(const BatchDrawEntry* d, const uint32_t* start, uint32_t nd,
                                                    unsigned long long* stats)
{
    __shared__ Material smat[256];
    const uint32_t mi = find_range(start, nd, blockIdx.x);
    const BatchDrawEntry& e = d[mi];
    for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < 256; i += blockDim.x * blockDim.y) smat[i] = e.mats[i];
    __syncthreads();
    const uint32_t local = blockIdx.x - start[mi];
    const uint32_t bx = local % e.gridX, by = local / e.gridX;
    Counters c;
    const uint32_t primary = draw_pixel(e.d, smat, bx * blockDim.x + threadIdx.x, by * blockDim.y + threadIdx.y, c);
    flush_counters(stats, c, primary, 0);
}

__global__ void __launch_bounds__(256) k_compact_batch(const CompactArgs* s, const uint32_t* start, uint32_t ns)
{
    const uint32_t mi = find_range(start, ns, blockIdx.x);
    compact_tiles(s[mi], (uint64_t)(blockIdx.x - start[mi]) * blockDim.x);
}

// blocks [0, nl): shadow directions of light map blockIdx.x.  Block nl: clamp the request count of every
// synced map to its capacity (dn_cuda_sync's k_clamp_requests), then the exclusive prefix of the light
// maps' counts into reqStart[0..nl] and a zero work counter.
__global__ void k_batch_prep(BatchLightMap* l, uint32_t nl, const CompactArgs* s, uint32_t ns, uint32_t* reqStart,
                             uint32_t* workCounter)
{
    if (blockIdx.x < nl) {
        BatchLightMap& e = l[blockIdx.x];
        for (int k = threadIdx.x; k < 65; k += blockDim.x) shadow_dir(e.p, k, e.sdir[k], e.sinv[k]);
        return;
    }
    for (uint32_t i = threadIdx.x; i < ns; i += blockDim.x) {
        uint32_t* c = &s[i].st->w[ST_REQ];
        if (*c > s[i].reqCap) *c = (uint32_t)s[i].reqCap;
    }
    __shared__ uint32_t warpSum[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) { carry = 0; *workCounter = 0; }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nl; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        uint32_t v = 0;
        if (i < nl) {
            v = *l[i].nreqPtr;
            if (v > l[i].reqCap) v = (uint32_t)l[i].reqCap;
        }
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if ((int)lane >= o) incl += t;
        }
        if (lane == 31u) warpSum[warp] = incl;
        __syncthreads();
        uint32_t before = carry;
        for (uint32_t w = 0; w < warp; w++) before += warpSum[w];
        if (i < nl) reqStart[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) reqStart[nl] = carry;
}

__global__ void __launch_bounds__(128, DN_STREAM_MIN_BLOCKS) k_light_stream_batch(const __grid_constant__ BatchLightArgs a)
{
    __shared__ Job jobs[128];
    stream_loop<true>(nullptr, &a, nullptr, jobs[threadIdx.x]);
}

// POOL: rays per fan kind per pool (the rays a warp pulls from a request group at a time); the autotuner
// picks PK_POOL_FAN or PK_POOL_ALT (dn_batch_tuning.poolRays)
template <uint32_t POOL>
__global__ void __launch_bounds__(128, DN_PACKET_MIN_BLOCKS) k_light_packet_batch(const __grid_constant__ BatchLightArgs a)
{
    __shared__ PacketWarpT<POOL> warps[4];
    packet_loop<true, POOL>(nullptr, &a, warps[threadIdx.x >> 5]);
}

// the opaque-chunk marks (mark_opaque_word) of every map of a lighting launch: block i marks map i
__global__ void __launch_bounds__(256) k_mark_opaque_batch(const BatchLightMap* l)
{
    __shared__ uint32_t opq[8];
    const BatchLightMap& e = l[blockIdx.x];
    opaque_materials(e.mats, opq);
    const uint64_t nwords = ((uint64_t)e.m.sx * e.m.sy * e.m.sz + 15) / 16;
    for (uint64_t wi = threadIdx.x; wi < nwords; wi += blockDim.x)
        mark_opaque_word(const_cast<uint32_t*>(e.m.tbits), e.m.tword, e.m.rec, wi, opq);
}

// the diffuse paths of the voxels k_light_packet_batch lit, as per-lane path streams over every map's queue
__global__ void __launch_bounds__(128, DN_DIFF_MIN_BLOCKS) k_light_diffuse_batch(const __grid_constant__ BatchLightArgs a)
{
    __shared__ Job jobs[128];
    stream_loop<true, true>(nullptr, &a, nullptr, jobs[threadIdx.x]);
}

__global__ void k_commit_batch(const BatchLightMap* l, const uint32_t* reqStart, uint32_t nl)
{
    const uint64_t total = (uint64_t)reqStart[nl] * 32u;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(i >> 5), lane = (uint32_t)(i & 31u);
        const uint32_t mi = find_range(reqStart, nl, r);
        const BatchLightMap& e = l[mi];
        const uint32_t lr = r - __ldg(&reqStart[mi]);
        commit_lane(e.m, e.reqs, e.out, (uint64_t)lr * 32u + lane, lr, lane, e.diffOut, e.specOut, e.samplesOut);
    }
}

// the status words of every member into one array (error flags are cleared once read)
__global__ void k_batch_gather(DevState* const* sts, uint32_t n, uint32_t* out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        DevState* s = sts[i];
        out[4 * i] = s->w[0]; out[4 * i + 1] = s->w[1]; out[4 * i + 2] = s->w[2]; out[4 * i + 3] = s->w[3];
        s->w[ST_ERR] = 0;
    }
}

// ------------------------------------------------------------------ host

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" int dn_cuda_batch_create(DNgpuBatch** out)
{
    if (!out) return dn_set_err(DN_CUDA_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (g_device < 0) return dn_set_err(DN_CUDA_ERR_DEVICE, "dn_cuda_init was not called");
    CK(cudaSetDevice(g_device));
    DNgpuBatch* b = new (std::nothrow) DNgpuBatch();
    if (!b) return dn_set_err(DN_CUDA_ERR_NOMEM, "host allocation");
    b->device = g_device;
    b->stream = b->side = nullptr;
    b->drawDone = b->copiesDone = b->tableFree = nullptr;
    b->htab = b->dtab = nullptr; b->tabCap = 0; b->tabGen = 0;
    b->workCounter = nullptr; b->bst = nullptr; b->hbst = nullptr; b->lsave = nullptr;
    b->dsts = nullptr; b->dstsCap = 0; b->stsDirty = true; b->dgather = nullptr; b->hgather = nullptr;
    b->gatherCount = 0;
    b->tuning.kernel = g_lightKernel == 2 ? 2u : 1u;
    b->tuning.streamBatch = b->tuning.kernel == 2u ? g_packetBatch : g_streamBatch;
    b->tuning.blocksPerSM = DN_STREAM_MIN_BLOCKS; b->tuning.useGraph = 1;
    b->tuning.poolRays = PK_POOL_FAN; b->tuning.diffuseBatch = g_streamBatch;
    b->lastPackets = false;
    b->graph = nullptr;
    b->lastLightValid = false;
    int rc = DN_CUDA_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->drawDone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->copiesDone, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->tableFree, cudaEventDisableTiming);
    if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "stream / event: %s", cudaGetErrorString(e));
    if (!rc) rc = dalloc(&b->workCounter, 1);
    if (!rc) rc = dalloc(&b->bst, 1);
    if (!rc) rc = dalloc(&b->lsave, 8);
    if (!rc) {
        COUNT_ALLOC();
        e = cudaMallocHost((void**)&b->hbst, sizeof(DevState));
        if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_NOMEM, "pinned: %s", cudaGetErrorString(e));
    }
    if (!rc) {
        e = cudaMemsetAsync(b->bst, 0, sizeof(DevState), b->stream);
        if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
    }
    if (!rc) {
        int perSM = 0, perSM2 = 0, perSM3 = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light_stream_batch, 128, 0);
        int perSMAlt = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM2, k_light_packet_batch<PK_POOL_FAN>, 128, 0);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSMAlt, k_light_packet_batch<PK_POOL_ALT>, 128, 0);
        b->maxBlocksPacketAlt = perSMAlt < 1 ? 1 : perSMAlt;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM3, k_light_diffuse_batch, 128, 0);
        if (e != cudaSuccess) rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "occupancy: %s", cudaGetErrorString(e));
        b->maxBlocksPerSM = perSM < 1 ? 1 : perSM;
        b->maxBlocksPacket = perSM2 < 1 ? 1 : perSM2;
        b->maxBlocksDiffuse = perSM3 < 1 ? 1 : perSM3;
        // every resident block the kernel allows
        b->tuning.blocksPerSM = (uint32_t)(b->tuning.kernel == 2u ? b->maxBlocksPacket : b->maxBlocksPerSM);
    }
    if (rc) { dn_cuda_batch_destroy(b); return rc; }
    *out = b;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_add(DNgpuBatch* b, DNgpuVolume* g)
{
    if (!b || !g) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (g->batch) return dn_set_err(DN_CUDA_ERR_ARG, "the volume already belongs to a batch");
    if (g->device != b->device) return dn_set_err(DN_CUDA_ERR_ARG, "the volume lives on another device");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(g->ownStream));
    g->stream = b->stream;
    g->batch = b;
    b->members.push_back(g);
    b->stsDirty = true;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_remove(DNgpuBatch* b, DNgpuVolume* g)
{
    if (!b || !g) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    auto it = std::find(b->members.begin(), b->members.end(), g);
    if (it == b->members.end() || g->batch != b) return dn_set_err(DN_CUDA_ERR_ARG, "the volume is not a member");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaStreamSynchronize(b->side));
    g->stream = g->ownStream;
    g->batch = nullptr;
    b->members.erase(it);
    b->stsDirty = true;
    b->lastKey.clear();
    b->lastLightValid = false;
    return DN_CUDA_OK;
}

extern "C" void dn_cuda_batch_destroy(DNgpuBatch* b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    while (!b->members.empty()) {
        DNgpuVolume* g = b->members.back();
        if (b->stream) cudaStreamSynchronize(b->stream);
        g->stream = g->ownStream;
        g->batch = nullptr;
        b->members.pop_back();
    }
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->side) cudaStreamSynchronize(b->side);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    dfree(b->dtab); dfree(b->workCounter); dfree(b->bst); dfree(b->lsave); dfree(b->dsts); dfree(b->dgather);
    if (b->htab) cudaFreeHost(b->htab);
    if (b->hbst) cudaFreeHost(b->hbst);
    if (b->hgather) cudaFreeHost(b->hgather);
    if (b->drawDone) cudaEventDestroy(b->drawDone);
    if (b->copiesDone) cudaEventDestroy(b->copiesDone);
    if (b->tableFree) cudaEventDestroy(b->tableFree);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// byte offsets of the sections of a frame's table
struct TableLayout {
    uint32_t nm, nd, ns, nl;
    size_t oMats, oDraw, oSync, oLight, oReqStart, oDrawStart, oSyncStart, size;
};

static TableLayout layout(uint32_t nm, uint32_t nd, uint32_t ns, uint32_t nl)
{
    TableLayout t;
    t.nm = nm; t.nd = nd; t.ns = ns; t.nl = nl;
    size_t o = 0;
    t.oMats = o; o = align256(o + (size_t)nm * 256 * sizeof(Material));
    t.oDraw = o; o = align256(o + (size_t)nd * sizeof(BatchDrawEntry));
    t.oSync = o; o = align256(o + (size_t)ns * sizeof(CompactArgs));
    t.oLight = o; o = align256(o + (size_t)nl * sizeof(BatchLightMap));
    t.oReqStart = o; o = align256(o + (size_t)(nl + 1) * 4);
    t.oDrawStart = o; o = align256(o + (size_t)(nd + 1) * 4);
    t.oSyncStart = o; o = align256(o + (size_t)(ns + 1) * 4);
    t.size = o;
    return t;
}

struct FramePlan {
    TableLayout t;
    uint32_t drawBlocks, syncBlocks;
    bool hostImages;
    bool packets;               // lighting as warp packets (dn_light_packet.cuh)
};

// packets: the lighting kernel of dn_light_packet.cuh (every map's specBounceLimit within its limit)
static int issue_light(DNgpuBatch* b, const BatchLightArgs& la, cudaStream_t s, bool packets)
{
    COUNT_LAUNCH();
    k_mark_opaque_batch<<<la.nmaps, 256, 0, s>>>(la.maps);
    CK(cudaGetLastError());
    COUNT_LAUNCH();
    const unsigned grid = (unsigned)(g_numSMs * (int)b->tuning.blocksPerSM);
    if (packets && b->tuning.poolRays == PK_POOL_ALT) k_light_packet_batch<PK_POOL_ALT><<<grid, 128, 0, s>>>(la);
    else if (packets) k_light_packet_batch<PK_POOL_FAN><<<grid, 128, 0, s>>>(la);
    else k_light_stream_batch<<<grid, 128, 0, s>>>(la);
    CK(cudaGetLastError());
    if (packets) {
        // the diffuse paths: a second pass over the same queue
        BatchLightArgs ld = la;
        ld.batch = b->tuning.diffuseBatch;
        CK(cudaMemsetAsync(la.workCounter, 0, 4, s));
        COUNT_LAUNCH();
        k_light_diffuse_batch<<<(unsigned)(g_numSMs * b->maxBlocksDiffuse), 128, 0, s>>>(ld);
        CK(cudaGetLastError());
    }
    return DN_CUDA_OK;
}

// the device work of one frame on b->stream; capturing: issued under stream capture
static int issue_frame(DNgpuBatch* b, const dn_batch_item* items, uint32_t n, const FramePlan& f, bool capturing)
{
    const TableLayout& t = f.t;
    cudaStream_t s = b->stream;
    unsigned char* d = b->dtab;
    const CompactArgs* syncs = (const CompactArgs*)(d + t.oSync);
    CK(cudaMemcpyAsync(d, b->htab, t.size, cudaMemcpyHostToDevice, s));
    // the host may rewrite its copy of the table once this fires (in a graph: an event record node)
    if (capturing) CK(cudaEventRecordWithFlags(b->tableFree, s, cudaEventRecordExternal));
    else CK(cudaEventRecord(b->tableFree, s));
    if (t.ns) {
        COUNT_LAUNCH();
        k_batch_reset<<<(t.ns + 255) / 256, 256, 0, s>>>(syncs, t.ns);
        CK(cudaGetLastError());
    }
    if (t.nd) {
        COUNT_LAUNCH();
        k_draw_batch<<<f.drawBlocks, dim3(8, 32), 0, s>>>((const BatchDrawEntry*)(d + t.oDraw),
                                                         (const uint32_t*)(d + t.oDrawStart), t.nd, b->bst->stats);
        CK(cudaGetLastError());
    }
    if (f.hostImages) {
        // host images: copies on the side stream overlap the rest of the frame
        CK(cudaEventRecord(b->drawDone, s));
        CK(cudaStreamWaitEvent(b->side, b->drawDone, 0));
        for (uint32_t i = 0; i < n; i++) {
            const dn_batch_item& it = items[i];
            if (!(it.phases & DN_BATCH_DRAW) || !it.hostImage) continue;
            const size_t px = (size_t)it.draw.width * it.draw.height;
            DNgpuVolume* g = it.map;
            CK(cudaMemcpyAsync(it.colorOut, g->dimg, px * 16, cudaMemcpyDeviceToHost, b->side));
            if (it.hitOut) CK(cudaMemcpyAsync(it.hitOut, g->dhit, px * 4, cudaMemcpyDeviceToHost, b->side));
            if (it.faceOut) CK(cudaMemcpyAsync(it.faceOut, g->dface, px, cudaMemcpyDeviceToHost, b->side));
        }
        CK(cudaEventRecord(b->copiesDone, b->side));
    }
    if (t.ns) {
        COUNT_LAUNCH();
        k_compact_batch<<<f.syncBlocks, 256, 0, s>>>(syncs, (const uint32_t*)(d + t.oSyncStart), t.ns);
        CK(cudaGetLastError());
    }
    if (t.nl || t.ns) {
        COUNT_LAUNCH();
        k_batch_prep<<<t.nl + 1, 128, 0, s>>>((BatchLightMap*)(d + t.oLight), t.nl, syncs, t.ns,
                                              (uint32_t*)(d + t.oReqStart), b->workCounter);
        CK(cudaGetLastError());
    }
    if (t.nl) {
        BatchLightArgs la;
        la.maps = (BatchLightMap*)(d + t.oLight);
        la.reqStart = (const uint32_t*)(d + t.oReqStart);
        la.nmaps = t.nl;
        la.workCounter = b->workCounter;
        la.stats = b->bst->lstats;
        la.batch = b->tuning.streamBatch;
        int rc = issue_light(b, la, s, f.packets);
        if (rc) return rc;
        COUNT_LAUNCH();
        k_commit_batch<<<(unsigned)(g_numSMs * 4), 256, 0, s>>>(la.maps, la.reqStart, t.nl);
        CK(cudaGetLastError());
        b->lastLight = la;
        b->lastLightValid = true;
        b->lastLightGens.clear();
        for (uint32_t i = 0; i < n; i++)
            if (items[i].phases & DN_BATCH_LIGHT) b->lastLightGens.emplace_back(items[i].map, items[i].map->gen);
    }
    if (f.hostImages) CK(cudaStreamWaitEvent(s, b->copiesDone, 0));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_frame(DNgpuBatch* b, const dn_batch_item* items, uint32_t n)
{
    if (!b || (!items && n)) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (n == 0) return DN_CUDA_OK;
    CK(cudaSetDevice(b->device));
    // validate, count sections, reserve image staging
    uint32_t nm = 0, nd = 0, ns = 0, nl = 0;
    bool hostImages = false;
    std::vector<const DNgpuVolume*> seen;
    seen.reserve(n);
    for (uint32_t i = 0; i < n; i++) {
        const dn_batch_item& it = items[i];
        DNgpuVolume* g = it.map;
        if (!g || g->batch != b) return dn_set_err(DN_CUDA_ERR_ARG, "item %u: the map is not a member of the batch", i);
        if (map_evicted(g)) return dn_set_err(DN_CUDA_ERR_ARG, "item %u: the map is evicted", i);
        if (!it.phases || (it.phases & ~(DN_BATCH_DRAW | DN_BATCH_SYNC | DN_BATCH_LIGHT)))
            return dn_set_err(DN_CUDA_ERR_ARG, "item %u: phases 0x%x", i, it.phases);
        seen.push_back(g);
        if (it.phases & (DN_BATCH_DRAW | DN_BATCH_LIGHT)) {
            if (!it.materials) return dn_set_err(DN_CUDA_ERR_ARG, "item %u: no materials", i);
            nm++;
        }
        if (it.phases & DN_BATCH_DRAW) {
            if (!it.colorOut || it.draw.width == 0 || it.draw.height == 0)
                return dn_set_err(DN_CUDA_ERR_ARG, "item %u: bad image", i);
            const int rc = dn_check_raster(&it.draw);
            if (rc) return rc;
            if (it.hostImage) {
                hostImages = true;
                int rc = dn_reserve_image_staging(g, (size_t)it.draw.width * it.draw.height);
                if (rc) return rc;
            }
            nd++;
        }
        if (it.phases & DN_BATCH_SYNC) {
            if (it.sync.split == 0 || it.sync.op > 2) return dn_set_err(DN_CUDA_ERR_ARG, "item %u: bad sync parameters", i);
            ns++;
        }
        if (it.phases & DN_BATCH_LIGHT) {
            if (it.light.K < 1 || it.light.K > 64) return dn_set_err(DN_CUDA_ERR_ARG, "item %u: K = %u", i, it.light.K);
            nl++;
        }
    }
    std::sort(seen.begin(), seen.end());
    if (std::adjacent_find(seen.begin(), seen.end()) != seen.end())
        return dn_set_err(DN_CUDA_ERR_ARG, "a map appears twice in one batched frame");

    FramePlan f;
    f.t = layout(nm, nd, ns, nl);
    f.hostImages = hostImages;
    uint32_t maxSpec = 0;
    for (uint32_t i = 0; i < n; i++)
        if ((items[i].phases & DN_BATCH_LIGHT) && items[i].light.specBounceLimit > maxSpec) maxSpec = items[i].light.specBounceLimit;
    f.packets = b->tuning.kernel == 2u && maxSpec <= PK_MAX_SPEC_SEGMENTS;
    b->lastPackets = f.packets;
    if (f.t.size > b->tabCap) {
        // growing waits for the stream, frees pinned memory (which waits for the device) and renews the
        // graph, a stall of up to two frames: the first table is large enough for about 370 maps per frame
        // (about 11 KB each, 8 KB of it materials), so a server whose ticks grow from a few maps to dozens
        // never grows it
        CK(cudaStreamSynchronize(b->stream));
        if (b->htab) cudaFreeHost(b->htab);
        b->htab = nullptr;
        dfree(b->dtab);
        const size_t minTable = (size_t)4 << 20;
        const size_t nc = f.t.size + f.t.size / 2 > minTable ? f.t.size + f.t.size / 2 : minTable;
        COUNT_ALLOC();
        CK(cudaMallocHost((void**)&b->htab, nc));
        int rc = dalloc(&b->dtab, nc);
        if (rc) { b->tabCap = 0; return rc; }
        b->tabCap = nc;
        b->tabGen++;
    }
    // the previous frame's copy of the table has been consumed once tableFree fired
    CK(cudaEventSynchronize(b->tableFree));
    unsigned char* h = b->htab;
    Material* hm = (Material*)(h + f.t.oMats);
    BatchDrawEntry* hd = (BatchDrawEntry*)(h + f.t.oDraw);
    CompactArgs* hs = (CompactArgs*)(h + f.t.oSync);
    BatchLightMap* hl = (BatchLightMap*)(h + f.t.oLight);
    uint32_t* drawStart = (uint32_t*)(h + f.t.oDrawStart);
    uint32_t* syncStart = (uint32_t*)(h + f.t.oSyncStart);
    const Material* dm = (const Material*)(b->dtab + f.t.oMats);
    uint32_t im = 0, id = 0, is = 0, il = 0, blocksD = 0, blocksS = 0;
    std::vector<uint64_t> key;
    key.reserve(4 + (size_t)n * 10);
    key.push_back(n); key.push_back(b->tabGen); key.push_back(b->tuning.streamBatch); key.push_back(b->tuning.blocksPerSM);
    key.push_back(b->tuning.kernel);
    for (uint32_t i = 0; i < n; i++) {
        const dn_batch_item& it = items[i];
        DNgpuVolume* g = it.map;
        key.push_back((uint64_t)(uintptr_t)g); key.push_back(g->gen); key.push_back(it.phases | (it.hostImage << 8));
        const Material* mats = nullptr;
        if (it.phases & (DN_BATCH_DRAW | DN_BATCH_LIGHT)) {
            memcpy(hm + (size_t)im * 256, it.materials, 256 * sizeof(Material));
            mats = dm + (size_t)im * 256;
            im++;
        }
        if (it.phases & DN_BATCH_DRAW) {
            BatchDrawEntry& e = hd[id];
            memset(&e, 0, sizeof(e));
            e.d.m = dev_map(g);
            e.d.m.degen = &b->bst->stats[S_DEGEN];
            e.d.p = it.draw;
            e.d.color = it.hostImage ? g->dimg : (float4*)it.colorOut;
            e.d.hit = it.hitOut ? (it.hostImage ? g->dhit : it.hitOut) : nullptr;
            e.d.face = it.faceOut ? (it.hostImage ? g->dface : it.faceOut) : nullptr;
            e.d.stats = b->bst->stats;
            e.mats = mats;
            e.gridX = (it.draw.width + 7) / 8;
            drawStart[id] = blocksD;
            blocksD += e.gridX * ((it.draw.height + 31) / 32);
            key.push_back((uint64_t)(uintptr_t)it.colorOut); key.push_back((uint64_t)(uintptr_t)it.hitOut);
            key.push_back((uint64_t)(uintptr_t)it.faceOut); key.push_back(((uint64_t)it.draw.width << 32) | it.draw.height);
            id++;
        }
        if (it.phases & DN_BATCH_SYNC) {
            CompactArgs& a = hs[is];
            memset(&a, 0, sizeof(a));
            a.tword = g->tword; a.tbits = g->tbits; a.treq = g->treq; a.tvis = g->tvis; a.ttouch = g->ttouch; a.tlast = g->tlast;
            a.tpend = g->tpend; a.tpendSlot = g->tpendSlot; a.rec = g->rec;
            a.reqs = g->reqs; a.reqCap = g->reqCap; a.st = g->st; a.ntiles = g->ntiles;
            a.op = it.sync.op; a.split = it.sync.split; a.frameNum = it.sync.frameNum;
            syncStart[is] = blocksS;
            blocksS += (uint32_t)((g->ntiles + 255) / 256);
            is++;
        }
        if (it.phases & DN_BATCH_LIGHT) {
            BatchLightMap& e = hl[il];
            memset(&e, 0, offsetof(BatchLightMap, sdir));
            e.m = dev_map(g);
            e.m.degen = &b->bst->lstats[S_DEGEN];
            e.reqs = g->reqs; e.nsamples = g->nsamples; e.out = g->lightOut;
            e.nreqPtr = &g->st->w[ST_REQ]; e.reqCap = g->reqCap;
            e.p = it.light;
            e.mats = mats;
            e.diffOut = g->diff; e.specOut = g->spec; e.samplesOut = g->nsamples;
            il++;
        }
    }
    drawStart[nd] = blocksD;
    syncStart[ns] = blocksS;
    f.drawBlocks = blocksD;
    f.syncBlocks = blocksS;

    const bool repeat = b->tuning.useGraph && key == b->lastKey;
    b->lastKey = key;
    if (!repeat) return issue_frame(b, items, n, f, false);
    if (!b->graph || b->graphKey != key) {
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        b->graphKey.clear();
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const unsigned long long before = g_launches;
        int rc = issue_frame(b, items, n, f, true);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
        __atomic_store_n(&g_launches, before, __ATOMIC_RELAXED);   // captured launches run when the graph does
        if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
        if (e != cudaSuccess) return dn_set_err(DN_CUDA_ERR_LAUNCH, "stream capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { b->graph = nullptr; return dn_set_err(DN_CUDA_ERR_LAUNCH, "graph instantiate: %s", cudaGetErrorString(e)); }
        b->graphKey = key;
    }
    // the graph's kernels: reset and compact (sync), draw, prep, light and commit
    const unsigned long long k = (f.t.ns ? 2u : 0u) + (f.t.nd ? 1u : 0u) + ((f.t.nl || f.t.ns) ? 1u : 0u) + (f.t.nl ? 2u : 0u);
    __atomic_fetch_add(&g_launches, k, __ATOMIC_RELAXED);
    CK(cudaGraphLaunch(b->graph, b->stream));
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_finish(DNgpuBatch* b)
{
    if (!b) return dn_set_err(DN_CUDA_ERR_ARG, "null batch");
    CK(cudaSetDevice(b->device));
    // the status blocks of the resident members only: an evicted map has none on the device, and a
    // restored one has it at a new address, so the pointer list is rebuilt whenever it changed
    std::vector<DNgpuVolume*> res;
    std::vector<DevState*> sts;
    for (DNgpuVolume* g : b->members)
        if (!g->evicted && g->st) { res.push_back(g); sts.push_back(g->st); }
    const uint32_t n = (uint32_t)res.size();
    if (n) {
        bool changed = b->stsDirty || n != b->gatherCount;
        if (!changed) changed = memcmp(b->gatherHost.data(), sts.data(), (size_t)n * sizeof(DevState*)) != 0;
        if (changed) {
            CK(cudaStreamSynchronize(b->stream));
            if (n > b->dstsCap) {
                dfree(b->dsts); dfree(b->dgather);
                if (b->hgather) cudaFreeHost(b->hgather);
                b->hgather = nullptr;
                b->dstsCap = 0;
                int rc;
                if ((rc = dalloc(&b->dsts, n)) || (rc = dalloc(&b->dgather, (size_t)n * 4))) return rc;
                COUNT_ALLOC();
                CK(cudaMallocHost((void**)&b->hgather, (size_t)n * 16));
                b->dstsCap = n;
            }
            CK(cudaMemcpy(b->dsts, sts.data(), (size_t)n * sizeof(DevState*), cudaMemcpyHostToDevice));
            b->gatherHost = sts;
            b->gatherCount = n;
            b->stsDirty = false;
        }
        COUNT_LAUNCH();
        k_batch_gather<<<(n + 255) / 256, 256, 0, b->stream>>>(b->dsts, n, b->dgather);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(b->hgather, b->dgather, (size_t)n * 16, cudaMemcpyDeviceToHost, b->stream));
    }
    CK(cudaMemcpyAsync(b->hbst, b->bst, sizeof(DevState), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaStreamSynchronize(b->side));
    uint32_t bad = 0, first = 0, flags = 0;
    for (uint32_t i = 0; i < n; i++) {
        DNgpuVolume* g = res[i];
        memcpy(g->hst->w, &b->hgather[4 * i], sizeof(g->hst->w));
        if (g->hst->w[ST_ERR]) { if (!bad) { first = i; flags = g->hst->w[ST_ERR]; } bad++; }
    }
    if (bad) return dn_set_err(DN_CUDA_ERR_KERNEL, "kernel error flags 0x%x on resident member %u (%u members flagged)", flags, first, bad);
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_stats(DNgpuBatch* b, int kind, dn_stats* out)
{
    if (!b || !out || kind < 0 || kind > 2) return dn_set_err(DN_CUDA_ERR_ARG, "bad argument");
    int rc = dn_cuda_batch_finish(b);
    if (rc && rc != DN_CUDA_ERR_KERNEL) return rc;
    unsigned long long s[8];
    for (int k = 0; k < 8; k++) s[k] = (kind != 2 ? b->hbst->stats[k] : 0ull) + (kind != 1 ? b->hbst->lstats[k] : 0ull);
    out->rays = s[S_RAYS]; out->primary = s[S_PRIMARY]; out->outerSteps = s[S_OUTER];
    out->chunksEntered = s[S_ENTERED]; out->innerSteps = s[S_INNER]; out->hits = s[S_HITS]; out->litVoxels = s[S_LIT];
    out->degenerate = s[S_DEGEN];
    return rc;
}

extern "C" int dn_cuda_batch_reset_stats(DNgpuBatch* b)
{
    if (!b) return dn_set_err(DN_CUDA_ERR_ARG, "null batch");
    CK(cudaSetDevice(b->device));
    CK(cudaMemsetAsync(b->bst->stats, 0, sizeof(b->bst->stats) + sizeof(b->bst->lstats), b->stream));
    return DN_CUDA_OK;
}

extern "C" void* dn_cuda_batch_stream(DNgpuBatch* b) { return b ? (void*)b->stream : nullptr; }

extern "C" int dn_cuda_batch_get_tuning(DNgpuBatch* b, dn_batch_tuning* out)
{
    if (!b || !out) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    *out = b->tuning;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_set_tuning(DNgpuBatch* b, const dn_batch_tuning* t)
{
    if (!b || !t) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    if (t->streamBatch < 1 || t->streamBatch > 32) return dn_set_err(DN_CUDA_ERR_ARG, "streamBatch %u", t->streamBatch);
    if (t->kernel != 1u && t->kernel != 2u) return dn_set_err(DN_CUDA_ERR_ARG, "kernel %u (1 streams, 2 packets)", t->kernel);
    if (t->poolRays != PK_POOL_FAN && t->poolRays != PK_POOL_ALT)
        return dn_set_err(DN_CUDA_ERR_ARG, "poolRays %u (%u or %u)", t->poolRays, PK_POOL_FAN, PK_POOL_ALT);
    if (t->diffuseBatch < 1 || t->diffuseBatch > 32) return dn_set_err(DN_CUDA_ERR_ARG, "diffuseBatch %u", t->diffuseBatch);
    const int maxBlocks = t->kernel == 2u ? (t->poolRays == PK_POOL_FAN ? b->maxBlocksPacket : b->maxBlocksPacketAlt)
                                          : b->maxBlocksPerSM;
    if (t->blocksPerSM < 1 || (int)t->blocksPerSM > maxBlocks)
        return dn_set_err(DN_CUDA_ERR_ARG, "blocksPerSM %u (1..%d)", t->blocksPerSM, maxBlocks);
    b->tuning = *t;
    b->tuning.useGraph = t->useGraph ? 1u : 0u;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_batch_autotune(DNgpuBatch* b, dn_batch_tuning* chosen)
{
    if (!b) return dn_set_err(DN_CUDA_ERR_ARG, "null batch");
    if (!b->lastLightValid) return dn_set_err(DN_CUDA_ERR_ARG, "no batched lighting launch to tune on");
    // the launch re-run names the maps' device arrays as they were at that frame
    for (const auto& mg : b->lastLightGens)
        if (mg.first->batch != b || mg.first->evicted || mg.first->gen != mg.second)
            return dn_set_err(DN_CUDA_ERR_ARG, "a map of the last batched frame changed since; run a frame before tuning");
    CK(cudaSetDevice(b->device));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // The reruns read the committed lighting and sample counts, so voxels lit for the first time in that
    // frame now trace their later-sample rays: the requested / touched / visible flags they set are saved
    // here and restored afterwards, as are the launch counters; the scratch they write is overwritten by
    // the next frame.
    CK(cudaMemcpyAsync(b->lsave, b->bst->lstats, sizeof(b->bst->lstats), cudaMemcpyDeviceToDevice, b->stream));
    size_t flagBytes = 0;
    for (const auto& mg : b->lastLightGens) flagBytes += 3 * mg.first->ntiles;
    unsigned char* saved = nullptr;
    COUNT_ALLOC();
    CK(cudaMalloc((void**)&saved, flagBytes ? flagBytes : 1));
    {
        size_t o = 0;
        for (const auto& mg : b->lastLightGens) {
            const DNgpuVolume* g = mg.first;
            CK(cudaMemcpyAsync(saved + o, g->treq, g->ntiles, cudaMemcpyDeviceToDevice, b->stream)); o += g->ntiles;
            CK(cudaMemcpyAsync(saved + o, g->ttouch, g->ntiles, cudaMemcpyDeviceToDevice, b->stream)); o += g->ntiles;
            CK(cudaMemcpyAsync(saved + o, g->tvis, g->ntiles, cudaMemcpyDeviceToDevice, b->stream)); o += g->ntiles;
        }
    }
    const dn_batch_tuning keep = b->tuning;
    dn_batch_tuning best = keep;
    // packets were possible in the last frame only if every lit map's specBounceLimit allowed them
    const bool packetsOk = b->lastPackets || keep.kernel != 2u;
    float bestMs = 3.4e38f;
    int rc = DN_CUDA_OK;
    // times the last frame's lighting launch under tuning t (best of two runs)
    auto trial = [&](const dn_batch_tuning& t) -> float {
        b->tuning = t;
        BatchLightArgs la = b->lastLight;
        la.batch = t.streamBatch;
        float ms = 3.4e38f;
        for (int rep = 0; rep < 2 && !rc; rep++) {
            cudaError_t e = cudaMemsetAsync(b->workCounter, 0, 4, b->stream);
            if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
            if (e != cudaSuccess) { rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "autotune: %s", cudaGetErrorString(e)); break; }
            rc = issue_light(b, la, b->stream, t.kernel == 2u && packetsOk);
            if (rc) break;
            e = cudaEventRecord(e1, b->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float t_ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t_ms, e0, e1);
            if (e != cudaSuccess) { rc = dn_set_err(DN_CUDA_ERR_LAUNCH, "autotune: %s", cudaGetErrorString(e)); break; }
            if (t_ms < ms) ms = t_ms;
        }
        if (!rc && ms < bestMs) { bestMs = ms; best = t; }
        return ms;
    };
    // coordinate descent: kernel, batch threshold, then resident blocks per SM
    trial(keep);
    {
        dn_batch_tuning t = best;
        t.kernel = 3u - t.kernel;
        t.streamBatch = t.kernel == 2u ? g_packetBatch : g_streamBatch;
        t.blocksPerSM = (uint32_t)(t.kernel == 2u ? b->maxBlocksPacket : b->maxBlocksPerSM);
        if (!rc && (t.kernel == 1u || packetsOk)) trial(t);
    }
    const uint32_t batches[] = {4u, 8u, 12u, 16u, 20u, 24u, 28u, 32u};
    for (uint32_t sb : batches) { dn_batch_tuning t = best; t.streamBatch = sb; if (!rc) trial(t); }
    if (best.kernel == 2u && packetsOk) {
        // rays a warp pulls per pool, then the diffuse kernel's refill threshold
        {
            dn_batch_tuning t = best;
            t.poolRays = best.poolRays == PK_POOL_FAN ? PK_POOL_ALT : PK_POOL_FAN;
            const uint32_t mx = (uint32_t)(t.poolRays == PK_POOL_FAN ? b->maxBlocksPacket : b->maxBlocksPacketAlt);
            if (t.blocksPerSM > mx) t.blocksPerSM = mx;
            if (!rc) trial(t);
        }
        const uint32_t dbatches[] = {8u, 12u, 16u, 20u, 24u, 28u};
        for (uint32_t db : dbatches) { dn_batch_tuning t = best; t.diffuseBatch = db; if (!rc) trial(t); }
    }
    const uint32_t bpsMax = (uint32_t)(best.kernel == 2u ? (best.poolRays == PK_POOL_FAN ? b->maxBlocksPacket
                                                                                    : b->maxBlocksPacketAlt)
                                                       : b->maxBlocksPerSM);
    for (uint32_t bps = 2; bps <= bpsMax && bps <= 8; bps++) {
        dn_batch_tuning t = best; t.blocksPerSM = bps; if (!rc) trial(t);
    }
    b->tuning = rc ? keep : best;
    b->tuning.useGraph = keep.useGraph;
    {
        size_t o = 0;
        for (const auto& mg : b->lastLightGens) {
            DNgpuVolume* g = mg.first;
            cudaMemcpyAsync(g->treq, saved + o, g->ntiles, cudaMemcpyDeviceToDevice, b->stream); o += g->ntiles;
            cudaMemcpyAsync(g->ttouch, saved + o, g->ntiles, cudaMemcpyDeviceToDevice, b->stream); o += g->ntiles;
            cudaMemcpyAsync(g->tvis, saved + o, g->ntiles, cudaMemcpyDeviceToDevice, b->stream); o += g->ntiles;
        }
    }
    cudaMemcpyAsync(b->bst->lstats, b->lsave, sizeof(b->bst->lstats), cudaMemcpyDeviceToDevice, b->stream);
    cudaStreamSynchronize(b->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(saved);
    if (rc) return rc;
    b->lastKey.clear();
    if (chosen) *chosen = b->tuning;
    return DN_CUDA_OK;
}

extern "C" uint64_t dn_cuda_requests_of(DNgpuVolume* g) { return g && g->hst ? g->hst->w[ST_REQ] : 0u; }
