/*
 * dn_cuda.cu -- CUDA kernels for sm_103a and the C ABI of include/dn_cuda.h.
 *
 * Device layout of one map (struct DNgpuVolume):
 *   tiles   tword[t] = state << 30 | record slot   (state 0 absent, 1 unloaded, 2 loaded)
 *           treq / tvis / ttouch (bytes), tlast (lastUsed), tpend / tpendSlot (host ops of a sync)
 *   records rec[slot]: 128-B ChunkRec (512-bit occupancy mask, partial counts, voxel count,
 *           position, pool base), nsamples[slot]
 *   pool    vox[i] (uint2: normal word, linear albedo word), diff[i] / spec[i] (float4, FP32)
 *   frame   reqs[] ((tile << 4) | group), lightOut[] (scratch: new lighting per request lane)
 * Kernels per frame: k_draw (primary rays), k_sync_stage + k_compact (DN_sync_gpu),
 * k_light + k_commit (DN_update_lighting).
 */
#include "dn_cuda.h"
#include "dn_device.cuh"
#include "dn_light.cuh"
#include "dn_light_stream.cuh"
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <stdlib.h>
#include <new>
#include <mutex>
#include <stdarg.h>

using namespace dn;

static_assert(sizeof(dn_material) == 32, "material layout");
static_assert(sizeof(Material) == 32, "material layout");
static_assert(sizeof(ChunkRec) == 128, "record layout");
static_assert(sizeof(dn_chunk_record) == 96, "record layout");

// ------------------------------------------------------------------ errors

static thread_local char t_err[512] = "";

static int set_err(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return set_err(e_ == cudaErrorMemoryAllocation ? DN_CUDA_ERR_NOMEM : DN_CUDA_ERR_LAUNCH, \
                           "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

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

// ------------------------------------------------------------------ state

enum { ST_REQ = 0, ST_WORK = 1, ST_ERR = 2 };
enum { S_RAYS = 0, S_PRIMARY, S_OUTER, S_ENTERED, S_INNER, S_HITS, S_LIT, S_COUNT };

struct DevState {
    uint32_t w[4];                      // nreq, work counter, error flags, pad
    unsigned long long stats[8];        // draw kernels
    unsigned long long lstats[8];       // lighting kernels
};

struct DNgpuVolume {
    int device;
    cudaStream_t stream;
    uint32_t sx, sy, sz;
    uint64_t ntiles;
    uint32_t* tword; uint8_t* treq; uint8_t* tvis; uint8_t* ttouch;
    uint32_t* tbits;                    // 2 bits per tile: 0 absent, 1 unloaded, 2 loaded (16 tiles per word)
    uint32_t* tlast; uint32_t* tpend; uint32_t* tpendSlot;
    ChunkRec* rec; uint32_t* nsamples; uint32_t slotCap;
    uint2* vox; float4* diff; float4* spec; uint64_t voxCap;
    uint32_t* reqs; float4* lightOut; uint64_t reqCap;
    DevState* st;
    // pinned staging for sync uploads and small readbacks
    unsigned char* hstage; size_t hstageCap;
    unsigned char* dstage; size_t dstageCap;
    cudaEvent_t stageFree;
    DevState* hst;                      // pinned copy of DevState
    // device staging for host-memory draws
    float4* dimg; uint32_t* dhit; uint8_t* dface; size_t dimgCap;
    int numSMs;
};

static int g_device = -1;
static int g_numSMs = 0;
static unsigned long long g_launches = 0;   // kernels launched by this library (all threads)
#define COUNT_LAUNCH() __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED)

extern "C" uint64_t dn_cuda_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

// lighting kernel selection and stream batch threshold (DN_LIGHT_KERNEL=0 lockstep, 1 streams;
// DN_STREAM_BATCH lanes, 1..32), read once at init
static int g_lightKernel = 1;
static uint32_t g_streamBatch = 24;

extern "C" int dn_cuda_init(int device)
{
    if (const char* e = getenv("DN_LIGHT_KERNEL")) g_lightKernel = atoi(e);
    if (const char* e = getenv("DN_STREAM_BATCH")) {
        int b = atoi(e);
        g_streamBatch = (uint32_t)(b < 1 ? 1 : (b > 32 ? 32 : b));
    }
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return set_err(DN_CUDA_ERR_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    }
    if (device < 0) CK(cudaGetDevice(&device));
    if (device >= n) return set_err(DN_CUDA_ERR_ARG, "device %d of %d", device, n);
    CK(cudaSetDevice(device));
    CK(cudaFree(0));
    CK(cudaDeviceGetAttribute(&g_numSMs, cudaDevAttrMultiProcessorCount, device));
    g_device = device;
    return DN_CUDA_OK;
}

extern "C" void dn_cuda_shutdown(void) { g_device = -1; }

template <class T> static int dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc((void**)p, count * sizeof(T)));
    return DN_CUDA_OK;
}
template <class T> static void dfree(T*& p) { if (p) cudaFree(p); p = nullptr; }

static int alloc_tiles(DNgpuVolume* g)
{
    uint64_t n = g->ntiles;
    int rc;
    if ((rc = dalloc(&g->tword, n)) || (rc = dalloc(&g->treq, n)) || (rc = dalloc(&g->tvis, n)) ||
        (rc = dalloc(&g->tbits, (n + 31) / 32 * 2)) ||
        (rc = dalloc(&g->ttouch, n)) || (rc = dalloc(&g->tlast, n)) || (rc = dalloc(&g->tpend, n)) ||
        (rc = dalloc(&g->tpendSlot, n)))
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

static void free_tiles(DNgpuVolume* g)
{
    dfree(g->tword); dfree(g->tbits); dfree(g->treq); dfree(g->tvis); dfree(g->ttouch); dfree(g->tlast); dfree(g->tpend); dfree(g->tpendSlot);
}

extern "C" void dn_cuda_map_destroy(DNgpuVolume* g)
{
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    free_tiles(g);
    dfree(g->rec); dfree(g->nsamples); dfree(g->vox); dfree(g->diff); dfree(g->spec);
    dfree(g->reqs); dfree(g->lightOut); dfree(g->st); dfree(g->dstage);
    dfree(g->dimg); dfree(g->dhit); dfree(g->dface);
    if (g->hstage) cudaFreeHost(g->hstage);
    if (g->hst) cudaFreeHost(g->hst);
    if (g->stageFree) cudaEventDestroy(g->stageFree);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

static int reserve_requests(DNgpuVolume* g, uint64_t cap)
{
    if (cap <= g->reqCap) return DN_CUDA_OK;
    uint64_t nc = g->reqCap ? g->reqCap : 1024;
    while (nc < cap) nc *= 2;
    CK(cudaStreamSynchronize(g->stream));
    dfree(g->reqs); dfree(g->lightOut);
    int rc;
    if ((rc = dalloc(&g->reqs, nc)) || (rc = dalloc(&g->lightOut, nc * 64))) { g->reqCap = 0; return rc; }
    g->reqCap = nc;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_map_create(uint32_t sx, uint32_t sy, uint32_t sz, uint32_t slotCap, uint64_t voxelCap,
                                  DNgpuVolume** out)
{
    if (!out) return set_err(DN_CUDA_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (g_device < 0) return set_err(DN_CUDA_ERR_DEVICE, "dn_cuda_init was not called");
    uint64_t n = (uint64_t)sx * sy * sz;
    if (n == 0 || n >= (1ull << 28)) return set_err(DN_CUDA_ERR_ARG, "map size %ux%ux%u", sx, sy, sz);
    DNgpuVolume* g = new (std::nothrow) DNgpuVolume();
    if (!g) return set_err(DN_CUDA_ERR_NOMEM, "host allocation");
    memset(g, 0, sizeof(*g));
    g->device = g_device;
    g->numSMs = g_numSMs;
    g->sx = sx; g->sy = sy; g->sz = sz; g->ntiles = n;
    int rc = DN_CUDA_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete g; return set_err(DN_CUDA_ERR_LAUNCH, "stream: %s", cudaGetErrorString(e)); }
    e = cudaEventCreateWithFlags(&g->stageFree, cudaEventDisableTiming);
    if (e != cudaSuccess) rc = set_err(DN_CUDA_ERR_LAUNCH, "event: %s", cudaGetErrorString(e));
    if (!rc) rc = alloc_tiles(g);
    if (!rc) rc = dalloc(&g->rec, slotCap);
    if (!rc) rc = dalloc(&g->nsamples, slotCap);
    if (!rc) rc = dalloc(&g->vox, voxelCap);
    if (!rc) rc = dalloc(&g->diff, voxelCap);
    if (!rc) rc = dalloc(&g->spec, voxelCap);
    if (!rc) rc = dalloc(&g->st, 1);
    if (!rc) rc = reserve_requests(g, 1024);
    if (!rc) {
        e = cudaMallocHost((void**)&g->hst, sizeof(DevState));
        if (e != cudaSuccess) rc = set_err(DN_CUDA_ERR_NOMEM, "pinned: %s", cudaGetErrorString(e));
    }
    if (!rc) {
        e = cudaMemsetAsync(g->st, 0, sizeof(DevState), g->stream);
        if (e != cudaSuccess) rc = set_err(DN_CUDA_ERR_LAUNCH, "memset: %s", cudaGetErrorString(e));
    }
    if (rc) { dn_cuda_map_destroy(g); return rc; }
    g->slotCap = slotCap ? slotCap : 1;
    g->voxCap = voxelCap ? voxelCap : 1;
    *out = g;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_map_resize(DNgpuVolume* g, uint32_t sx, uint32_t sy, uint32_t sz)
{
    if (!g) return set_err(DN_CUDA_ERR_ARG, "null volume");
    uint64_t n = (uint64_t)sx * sy * sz;
    if (n == 0 || n >= (1ull << 28)) return set_err(DN_CUDA_ERR_ARG, "map size %ux%ux%u", sx, sy, sz);
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    free_tiles(g);
    g->sx = sx; g->sy = sy; g->sz = sz; g->ntiles = n;
    return alloc_tiles(g);
}

template <class T> static int grow_copy(DNgpuVolume* g, T** p, uint64_t oldCount, uint64_t newCount)
{
    T* np = nullptr;
    int rc = dalloc(&np, newCount);
    if (rc) return rc;
    if (*p && oldCount) CK(cudaMemcpyAsync(np, *p, oldCount * sizeof(T), cudaMemcpyDeviceToDevice, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    dfree(*p);
    *p = np;
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_reserve(DNgpuVolume* g, uint32_t slotCap, uint64_t voxelCap, uint64_t requestCap)
{
    if (!g) return set_err(DN_CUDA_ERR_ARG, "null volume");
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

// ------------------------------------------------------------ counters

__device__ __forceinline__ uint32_t lane_id()
{
    uint32_t l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

__device__ __forceinline__ void flush_counters(unsigned long long* stats, const Counters& c, uint32_t primary, uint32_t lit)
{
    // warp-reduce then one atomic per counter per warp
    uint32_t v[7] = {c.rays, primary, c.outer, c.entered, c.inner, c.hits, lit};
    const unsigned full = __activemask();
#pragma unroll
    for (int k = 0; k < 7; k++) {
        uint32_t x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(full, x, o);
        v[k] = x;
    }
    int leader = __ffs(full) - 1;
    if ((int)lane_id() == leader) {
#pragma unroll
        for (int k = 0; k < 7; k++) if (v[k]) atomicAdd(&stats[k], (unsigned long long)v[k]);
    }
}

// ------------------------------------------------------------------ draw

struct DrawArgs {
    DevMap m;
    dn_draw_params p;
    float4* color;
    uint32_t* hit;
    uint8_t* face;
    unsigned long long* stats;
    Material mats[256];
};

__global__ void __launch_bounds__(256) k_draw(const __grid_constant__ DrawArgs a)
{
    __shared__ Material smat[256];
    for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < 256; i += blockDim.x * blockDim.y) smat[i] = a.mats[i];
    __syncthreads();
    const dn_draw_params& p = a.p;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    RayCtx c;
    c.m = &a.m; c.mats = smat;
    c.sunStrength = mk(p.sunStrength[0], p.sunStrength[1], p.sunStrength[2]);
    c.emissive = p.emissiveStrength;
    c.refraction = true;   // voxelDraw.comp:65
    c.c = Counters{0, 0, 0, 0, 0};
    uint32_t primary = 0;
    if (x < p.width && y < p.height) {
        const uint64_t pix = (uint64_t)y * p.width + x;
        uint32_t hitIdx = 0xFFFFFFFFu;
        uint8_t face = 6;
        float4 out;
        const uint32_t limW = p.truncate16 ? (p.width / 16u) * 16u : p.width;
        const uint32_t limH = p.truncate16 ? (p.height / 16u) * 16u : p.height;
        if (x >= limW || y >= limH) {
            out = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        } else {
            const float sx = (float)x / (float)p.width * 2.0f - 1.0f;
            const float sy = (float)y / (float)p.height * 2.0f - 1.0f;
            f3 rayPos = mk(p.origin[0], p.origin[1], p.origin[2]);
            c.orgRayPos = rayPos;
            const float (*M)[4] = p.dirMat;
            f3 rd = mk(M[0][0] * sx + M[1][0] * sy + M[2][0] * 0.0f + M[3][0] * 1.0f,
                       M[0][1] * sx + M[1][1] * sy + M[2][1] * 0.0f + M[3][1] * 1.0f,
                       M[0][2] * sx + M[1][2] * sy + M[2][2] * 0.0f + M[3][2] * 1.0f);
            f3 rayDir = adds(normalize(rd), EPS);
            f3 inv = mk(1.0f / rayDir.x, 1.0f / rayDir.y, 1.0f / rayDir.z);
            const float maxDepth = -1.0f;
            const f3 mapMax = mk((float)a.m.sx, (float)a.m.sy, (float)a.m.sz);
            const f3 skyBot = mk(p.skyBot[0], p.skyBot[1], p.skyBot[2]), skyTop = mk(p.skyTop[0], p.skyTop[1], p.skyTop[2]);
            // intersect_AABB, voxelShared.comp:261-273
            f3 tMin = mul(sub(mk(0.0f, 0.0f, 0.0f), rayPos), inv);
            f3 tMax = mul(sub(mapMax, rayPos), inv);
            f3 t1 = mk(gmin(tMin.x, tMax.x), gmin(tMin.y, tMax.y), gmin(tMin.z, tMax.z));
            f3 t2 = mk(gmax(tMin.x, tMax.x), gmax(tMin.y, tMax.y), gmax(tMin.z, tMax.z));
            float tNear = gmax(gmax(t1.x, t1.y), t1.z);
            float tFar = gmin(gmin(t2.x, t2.y), t2.z);
            f3 fc;
            float depth = -1.0f;
            if (tNear > tFar || tFar < 0.0f) {
                f3 s = sky_color(skyBot, skyTop, rayDir);
                fc = mk(powf(s.x, 2.2f), powf(s.y, 2.2f), powf(s.z, 2.2f));
            } else {
                if (tNear > 0.0f) rayPos = add(rayPos, muls(rayDir, tNear + EPS));
                // normal_AABB, voxelShared.comp:276-284
                f3 cc = muls(add(mk(0.0f, 0.0f, 0.0f), mapMax), 0.5f);
                f3 pp = sub(rayPos, cc);
                f3 dd = muls(sub(mapMax, mk(0.0f, 0.0f, 0.0f)), 0.5f);
                const float bias = 1.0f + EPS;
                f3 q = mk(pp.x / dd.x * bias, pp.y / dd.y * bias, pp.z / dd.z * bias);
                f3 hitNormal = normalize(mk(truncf(q.x), truncf(q.y), truncf(q.z)));
                TState ts{255u, 1.0f};
                Voxel fv;
                fv.normal = mk(0.0f, 0.0f, 0.0f); fv.material = 0; fv.albedo = fv.normal; fv.spec = fv.normal; fv.diff = fv.normal;
                f3 cadd; float cmul; HitInfo hi;
                primary = 1;
                if (step_map(c, ts, rayDir, inv, rayPos, false, maxDepth, hitNormal, fv, cadd, cmul, hi)) {
                    i3 mp{f2i(floorf(rayPos.x)), f2i(floorf(rayPos.y)), f2i(floorf(rayPos.z))};
                    if (in_map(a.m, mp)) {
                        uint8_t* vp = &a.m.tvis[map_index(a.m, mp)];
                        if (*vp == 0) *vp = 1;
                    }
                    f3 dv = sub(rayPos, c.orgRayPos);
                    depth = sqrtf(dot(dv, dv));
                    // voxel_color, voxelDraw.comp:32-61
                    const Material& mt = smat[fv.material];
                    f3 sp = muls(fv.spec, mt.specular);
                    f3 df = muls(fv.diff, 1.0f - mt.specular);
                    switch (p.viewMode) {
                    case 0: {
                        f3 solid = mt.emissive ? muls(fv.albedo, c.emissive) : add(mul(df, fv.albedo), sp);
                        fc = add(muls(solid, cmul), cadd);
                        break;
                    }
                    case 1: fc = fv.albedo; break;
                    case 2: fc = mt.emissive ? fv.albedo : df; break;
                    case 3: fc = mt.emissive ? fv.albedo : sp; break;
                    case 4: fc = vabs(fv.normal); break;
                    case 5: fc = vabs(hitNormal); break;
                    default: fc = mk(0.0f, 0.0f, 0.0f); break;
                    }
                    const uint32_t tx = hi.tile % a.m.sx, ty = (hi.tile / a.m.sx) % a.m.sy, tz = hi.tile / (a.m.sx * a.m.sy);
                    const uint32_t gx = tx * 8u + (uint32_t)hi.local.x, gy = ty * 8u + (uint32_t)hi.local.y,
                                   gz = tz * 8u + (uint32_t)hi.local.z;
                    hitIdx = gx + (a.m.sx * 8u) * (gy + (a.m.sy * 8u) * gz);
                    if (hitNormal.x > 0.0f) face = 0; else if (hitNormal.x < 0.0f) face = 1;
                    else if (hitNormal.y > 0.0f) face = 2; else if (hitNormal.y < 0.0f) face = 3;
                    else if (hitNormal.z > 0.0f) face = 4; else if (hitNormal.z < 0.0f) face = 5;
                } else {
                    f3 s = sky_color(skyBot, skyTop, rayDir);
                    f3 bg = mk(powf(s.x, 2.2f), powf(s.y, 2.2f), powf(s.z, 2.2f));
                    fc = add(muls(bg, cmul), cadd);
                    depth = maxDepth;
                }
            }
            out = make_float4(powf(fc.x, 0.4545f), powf(fc.y, 0.4545f), powf(fc.z, 0.4545f), depth);
        }
        a.color[pix] = out;
        if (a.hit) a.hit[pix] = hitIdx;
        if (a.face) a.face[pix] = face;
    }
    flush_counters(a.stats, c.c, primary, 0);
}

// -------------------------------------------------------------- lighting

struct LightArgs {
    DevMap m;
    const uint32_t* reqs;
    DevState* st;
    const uint32_t* nsamples;
    float4* out;                // 2 float4 per request lane: diffuse, specular
    dn_light_params p;
    Material mats[256];
};

__global__ void __launch_bounds__(128) k_light(const __grid_constant__ LightArgs a)
{
    __shared__ Material smat[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) smat[i] = a.mats[i];
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    LightCtx L;
    L.rc.m = &a.m; L.rc.mats = smat;
    L.rc.sunStrength = mk(a.p.sunStrength[0], a.p.sunStrength[1], a.p.sunStrength[2]);
    L.rc.emissive = a.p.emissiveStrength;
    L.rc.refraction = false;   // voxelLighting.comp:209
    L.rc.orgRayPos = mk(0.0f, 0.0f, 0.0f);
    L.rc.c = Counters{0, 0, 0, 0, 0};
    L.p = &a.p;
    L.sunDir = mk(a.p.sunDir[0], a.p.sunDir[1], a.p.sunDir[2]);
    L.ambient = mk(a.p.ambient[0], a.p.ambient[1], a.p.ambient[2]);
    L.camPos = mk(a.p.camPos[0], a.p.camPos[1], a.p.camPos[2]);
    L.skyBot = mk(a.p.skyBot[0], a.p.skyBot[1], a.p.skyBot[2]);
    L.skyTop = mk(a.p.skyTop[0], a.p.skyTop[1], a.p.skyTop[2]);
    L.rngSin = a.p.rngMode == 1u;
    L.sample = 0;
    uint32_t lit = 0;
    const uint32_t nreq = *(volatile uint32_t*)&a.st->w[ST_REQ];
    while (true) {
        uint32_t r = 0;
        if (lane == 0) r = atomicAdd(&a.st->w[ST_WORK], 1u);
        r = __shfl_sync(0xFFFFFFFFu, r, 0);
        if (r >= nreq) break;
        const uint32_t word = a.reqs[r];
        const uint32_t tile = word >> 4, group = word & 15u;
        const uint32_t tw = __ldg(&a.m.tword[tile]);
        // every lane of the warp takes part (the phases use warp votes); lanes without a voxel idle
        bool active = false;
        i3 cp{0, 0, 0}, mp{0, 0, 0};
        uint32_t samples = 0;
        Voxel tv;
        tv.normal = mk(0.0f, 1.0f, 0.0f); tv.material = 0; tv.albedo = mk(0.0f, 0.0f, 0.0f);
        tv.spec = tv.albedo; tv.diff = tv.albedo;
        if ((tw >> 30) == 2u) {
            const uint32_t slot = tw & SLOT_MASK;
            const ChunkRec* rc = &a.m.rec[slot];
            const uint32_t vn = group * 32u + lane;
            uint32_t li;
            if (vn < __ldg(&rc->nvox) && select_voxel(rc, vn, cp, li)) {
                mp = i3{__ldg(&rc->pos[0]), __ldg(&rc->pos[1]), __ldg(&rc->pos[2])};
                decompress(a.m, __ldg(&rc->voxBase) + vn, tv);
                samples = __ldg(&a.nsamples[slot]);
                active = true;
            }
        }
        float4 od = make_float4(0.0f, 0.0f, 0.0f, 0.0f), os = od;
        light_voxel(L, active, mp, cp, tv, samples, od, os);
        if (!active) { od = make_float4(0.0f, 0.0f, 0.0f, 0.0f); os = od; }
        lit += active ? 1u : 0u;
        a.out[((uint64_t)r * 32u + lane) * 2u] = od;
        a.out[((uint64_t)r * 32u + lane) * 2u + 1u] = os;
    }
    flush_counters(a.st->lstats, L.rc.c, 0, lit);
}

#ifndef DN_STREAM_MIN_BLOCKS
#define DN_STREAM_MIN_BLOCKS 4   // 4 blocks of 4 warps per SM (measured best: leaves L1 room for the tile map)
#endif

// The lighting launch as persistent per-lane ray streams (dn_light_stream.cuh).
__global__ void __launch_bounds__(128, DN_STREAM_MIN_BLOCKS) k_light_stream(const __grid_constant__ StreamArgs a)
{
    __shared__ StreamShared sh;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sh.mats[i] = a.mats[i];
    {
        // shadow directions: normalize(sunDir * softness + P_k) + EPS and their reciprocals (identical for every voxel)
        const dn_light_params& p = a.p;
        const f3 sd = mk(p.sunDir[0], p.sunDir[1], p.sunDir[2]);
        for (int k = threadIdx.x; k < 65; k += blockDim.x) {
            f3 d;
            if (k == 64) d = adds(sd, EPS);
            else if ((uint32_t)k < p.K) {
                const f3 P = mk(p.spherePts[k][0], p.spherePts[k][1], p.spherePts[k][2]);
                d = adds(normalize(add(muls(sd, p.shadowSoftness), P)), EPS);
            } else d = mk(1.0f, 1.0f, 1.0f);
            sh.sdir[k][0] = d.x; sh.sdir[k][1] = d.y; sh.sdir[k][2] = d.z;
            sh.sinv[k][0] = __frcp_rn(d.x); sh.sinv[k][1] = __frcp_rn(d.y); sh.sinv[k][2] = __frcp_rn(d.z);
        }
    }
    __syncthreads();
    const uint32_t lane = lane_id();
    const uint32_t nreq = *(volatile const uint32_t*)a.nreqPtr;
    const f3 sun = mk(a.p.sunStrength[0], a.p.sunStrength[1], a.p.sunStrength[2]);
    const uint32_t batch = a.batch;
    uint32_t winReq = 0, winNext = 32;     // warp-uniform voxel window: request index, next lane in it
    bool exhausted = false;
    // per-voxel job state lives in shared memory: it is touched only when a segment ends
    __shared__ Job jobs[128];
    Job& j = jobs[threadIdx.x];
    j.phase = PH_FETCH;
    Seg s;
    bool rayActive = false;
    uint32_t hitState = 0, hitIdx = 0;
    Counters c{0, 0, 0, 0, 0};
    uint32_t lit = 0;
    while (true) {
        const unsigned waiting = __ballot_sync(0xFFFFFFFFu, !rayActive && j.phase != PH_DONE);
        const unsigned stepping = __ballot_sync(0xFFFFFFFFu, rayActive);
        if (waiting == 0u && stepping == 0u) break;
        if (stepping == 0u || (uint32_t)__popc(waiting) >= batch) {
            for (int round = 0; round < 4; round++) {
                // warp-cooperative voxel fetch for lanes whose voxel is done
                for (int guard = 0; guard < 64; guard++) {
                    const unsigned need = __ballot_sync(0xFFFFFFFFu, j.phase == PH_FETCH);
                    if (need == 0u) break;
                    if (winNext >= 32u) {
                        uint32_t r = 0;
                        if (!exhausted && lane == 0) r = atomicAdd(a.workCounter, 1u);
                        r = __shfl_sync(0xFFFFFFFFu, r, 0);
                        if (exhausted || r >= nreq) {
                            exhausted = true;
                            if (j.phase == PH_FETCH) j.phase = PH_DONE;
                            break;
                        }
                        winReq = r;
                        winNext = 0;
                    }
                    const uint32_t rank = __popc(need & ((1u << lane) - 1u));
                    if (j.phase == PH_FETCH && winNext + rank < 32u) voxel_setup(j, winReq, winNext + rank, a, sh);
                    const uint32_t took = (uint32_t)__popc(need) < 32u - winNext ? (uint32_t)__popc(need) : 32u - winNext;
                    winNext += took;
                }
                // shade the finished segment and set up the next one (or finish the voxel)
                if (!rayActive && j.phase != PH_DONE && j.phase != PH_FETCH)
                    rayActive = advance(j, s, hitState, hitIdx, a, sh, c, lit);
                if (__ballot_sync(0xFFFFFFFFu, j.phase == PH_FETCH) == 0u) break;
            }
        }
        if (rayActive) {
            const uint32_t r = seg_step(s, a.m, sh.mats, sun, c, hitIdx);
            if (r) { rayActive = false; hitState = r; }
        }
    }
    flush_counters(a.stats, c, 0, lit);
}

// D1/D2: commit the new lighting after the whole launch, then count the sample
__global__ void k_commit(DevMap m, const uint32_t* reqs, const DevState* st, const float4* out,
                         float4* diff, float4* spec, uint32_t* nsamples)
{
    const uint32_t nreq = st->w[ST_REQ];
    const uint64_t total = (uint64_t)nreq * 32u;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(i >> 5), lane = (uint32_t)(i & 31u);
        const uint32_t word = reqs[r];
        const uint32_t tile = word >> 4, group = word & 15u;
        const uint32_t tw = m.tword[tile];
        if ((tw >> 30) != 2u) continue;
        const uint32_t slot = tw & SLOT_MASK;
        const ChunkRec* rc = &m.rec[slot];
        const uint32_t vn = group * 32u + lane;
        if (vn >= rc->nvox) continue;
        const uint32_t idx = rc->voxBase + vn;
        diff[idx] = out[i * 2u];
        spec[idx] = out[i * 2u + 1u];
        if (vn == 0) nsamples[slot] += 1u;
    }
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
        if (op.tile >= ntiles) { if (threadIdx.x == 0) atomicOr(&st->w[ST_ERR], 1u); continue; }
        const bool staged = (op.flags & DN_PEND_STAGED) != 0;
        const dn_chunk_record* srcp = staged ? &recs[op.recordIndex] : nullptr;
        const bool bad = staged && (op.slot >= slotCap || srcp->nvox > 512u || (uint64_t)srcp->voxBase + srcp->nvox > voxCap);
        if (threadIdx.x == 0) {
            // a record that does not fit is not published: the tile stays unloaded
            tpend[op.tile] = bad ? (op.flags & ~DN_PEND_STAGED) : op.flags;
            tpendSlot[op.tile] = bad ? DN_SLOT_NONE : op.slot;
            if (bad) atomicOr(&st->w[ST_ERR], 2u);
        }
        if (!staged || bad) continue;
        const dn_chunk_record& src = *srcp;
        ChunkRec* dst = &rec[op.slot];
        const uint32_t* s32 = (const uint32_t*)&src;
        uint32_t* d32 = (uint32_t*)dst;
        if (threadIdx.x < 24) d32[threadIdx.x] = s32[threadIdx.x];
        if (threadIdx.x == 0) nsamples[op.slot] = 0;
        const uint64_t off = voxOff[op.recordIndex];
        for (uint32_t i = threadIdx.x; i < src.nvox; i += blockDim.x) {
            const uint64_t d = (uint64_t)src.voxBase + i;
            vox[d] = make_uint2(words[2 * (off + i)], words[2 * (off + i) + 1]);
            diff[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            spec[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// spreads the 16 low bits of x to the even bit positions of a word
__device__ __forceinline__ uint32_t spread_bits(uint32_t x)
{
    x &= 0xFFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

struct CompactArgs {
    uint32_t* tword; uint8_t* treq; uint8_t* tvis; uint8_t* ttouch; uint32_t* tlast;
    uint32_t* tbits;
    uint32_t* tpend; const uint32_t* tpendSlot;
    const ChunkRec* rec;
    uint32_t* reqs; uint64_t reqCap;
    DevState* st;
    uint64_t ntiles;
    uint32_t op, split, frameNum;
};

// the per-tile loop of DN_sync_gpu (voxel.c:738-762) with the request rule of
// _DN_request_chunk_lighting (1463-1489) and the state machine of _DN_stream_to_gpu (1491-1536)
__global__ void __launch_bounds__(256) k_compact(const __grid_constant__ CompactArgs a)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < a.ntiles; base += stride) {
        const uint64_t t = base + threadIdx.x;
        uint32_t groups = 0;
        uint32_t finalSt = 0;
        if (t < a.ntiles) {
            const uint32_t w = a.tword[t];
            const uint32_t st = w >> 30;
            finalSt = st;
            uint32_t slot = w & SLOT_MASK;
            const uint32_t pend = a.tpend[t];
            const bool req = a.treq[t] != 0;
            uint32_t vis = a.tvis[t];
            uint32_t gflag = (st == 1u && req) ? 3u : st;
            const bool updated = (pend & DN_PEND_UPDATED) != 0;
            uint32_t lu = a.tlast[t];
            if (a.ttouch[t]) { lu = 0; a.ttouch[t] = 0; }
            if (lu != 0xFFFFFFFFu) lu++;
            if (a.op != 1u && gflag == 2u && vis && (((uint32_t)t % a.split) == a.frameNum || updated)) {
                groups = (a.rec[slot].nvox + 31u) / 32u;
                vis = 0;
            }
            if (a.op != 0u) {
                const bool valid = (pend & DN_PEND_VALID) != 0;
                const bool exists = valid ? (pend & DN_PEND_EXISTS) != 0 : (st != 0u);
                const uint32_t newSlot = (pend & DN_PEND_STAGED) ? a.tpendSlot[t] : (valid ? DN_SLOT_NONE : slot);
                bool changed = false;
                if (exists && gflag == 0u) { gflag = 1u; changed = true; }
                else if (!exists && gflag != 0u) { gflag = 0u; changed = true; }
                if (gflag == 2u && updated) { gflag = 3u; changed = true; }
                if (gflag == 3u && exists && newSlot != DN_SLOT_NONE) { gflag = 2u; lu = 0; changed = true; }
                if (changed) vis = 0;
                slot = exists ? newSlot : DN_SLOT_NONE;
                a.treq[t] = (gflag == 3u) ? 1 : 0;
                finalSt = gflag == 3u ? 1u : gflag;
                a.tword[t] = (finalSt << 30) | (slot & SLOT_MASK);
            }
            if (pend) a.tpend[t] = 0;
            a.tvis[t] = (uint8_t)vis;
            a.tlast[t] = lu;
        }
        // the 2-bit tile map read by the chunk-level DDA step: 32 tiles per warp, two words
        {
            const unsigned b0 = __ballot_sync(0xFFFFFFFFu, finalSt == 1u);
            const unsigned b1 = __ballot_sync(0xFFFFFFFFu, finalSt == 2u);
            if (lane == 0 && base + threadIdx.x - lane < a.ntiles) {
                const uint64_t wi = (base + threadIdx.x) >> 4;
                a.tbits[wi] = spread_bits(b0 & 0xFFFFu) | (spread_bits(b1 & 0xFFFFu) << 1);
                a.tbits[wi + 1] = spread_bits(b0 >> 16) | (spread_bits(b1 >> 16) << 1);
            }
        }
        // warp-aggregated append of (tile << 4 | group) request words
        uint32_t incl = groups;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if ((int)lane >= o) incl += v;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        uint32_t wbase = 0;
        if (lane == 31 && total) wbase = atomicAdd(&a.st->w[ST_REQ], total);
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 31);
        if (groups) {
            const uint32_t first = wbase + incl - groups;
            for (uint32_t gi = 0; gi < groups; gi++) {
                if ((uint64_t)first + gi < a.reqCap) a.reqs[first + gi] = ((uint32_t)t << 4) | gi;
                else atomicOr(&a.st->w[ST_ERR], 4u);
            }
        }
    }
}

__global__ void k_clamp_requests(DevState* st, uint64_t cap)
{
    if (st->w[ST_REQ] > cap) st->w[ST_REQ] = (uint32_t)cap;
}

extern "C" int dn_cuda_sync(DNgpuVolume* g, const dn_sync_params* p, const dn_tile_op* ops, uint32_t nops,
                            const dn_chunk_record* records, uint32_t nrecords, const uint32_t* voxelWords,
                            uint64_t nvoxels)
{
    if (!g || !p) return set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->split == 0 || p->op > 2) return set_err(DN_CUDA_ERR_ARG, "bad sync parameters");
    CK(cudaSetDevice(g->device));
    if (nops) {
        // one pinned upload: ops | records | voxel offsets | voxel words
        const size_t bOps = (size_t)nops * sizeof(dn_tile_op);
        const size_t bRec = (size_t)nrecords * sizeof(dn_chunk_record);
        const size_t bOff = (size_t)nrecords * sizeof(uint64_t);
        const size_t bVox = (size_t)nvoxels * 8u;
        const size_t oRec = (bOps + 15) & ~(size_t)15, oOff = (oRec + bRec + 15) & ~(size_t)15,
                     oVox = (oOff + bOff + 15) & ~(size_t)15, total = oVox + bVox;
        CK(cudaEventSynchronize(g->stageFree));
        if (total > g->hstageCap) {
            if (g->hstage) cudaFreeHost(g->hstage);
            g->hstage = nullptr;
            size_t nc = total + total / 2 + 4096;
            CK(cudaMallocHost((void**)&g->hstage, nc));
            g->hstageCap = nc;
        }
        if (total > g->dstageCap) {
            CK(cudaStreamSynchronize(g->stream));
            dfree(g->dstage);
            size_t nc = total + total / 2 + 4096;
            int rc = dalloc(&g->dstage, nc);
            if (rc) { g->dstageCap = 0; return rc; }
            g->dstageCap = nc;
        }
        memcpy(g->hstage, ops, bOps);
        if (bRec) memcpy(g->hstage + oRec, records, bRec);
        uint64_t* off = (uint64_t*)(g->hstage + oOff);
        uint64_t acc = 0;
        for (uint32_t r = 0; r < nrecords; r++) { off[r] = acc; acc += records[r].nvox; }
        if (acc != nvoxels) return set_err(DN_CUDA_ERR_ARG, "voxel word count %llu != %llu", (unsigned long long)acc, (unsigned long long)nvoxels);
        for (uint32_t o = 0; o < nops; o++)
            if ((ops[o].flags & DN_PEND_STAGED) && ops[o].recordIndex >= nrecords)
                return set_err(DN_CUDA_ERR_ARG, "op %u references record %u of %u", o, ops[o].recordIndex, nrecords);
        if (bVox) memcpy(g->hstage + oVox, voxelWords, bVox);
        CK(cudaMemcpyAsync(g->dstage, g->hstage, total, cudaMemcpyHostToDevice, g->stream));
        CK(cudaEventRecord(g->stageFree, g->stream));
        COUNT_LAUNCH();
        k_sync_stage<<<nops < 65535u ? nops : 65535u, 128, 0, g->stream>>>(
            (const dn_tile_op*)g->dstage, nops, (const dn_chunk_record*)(g->dstage + oRec),
            (const uint64_t*)(g->dstage + oOff), (const uint32_t*)(g->dstage + oVox), g->tpend, g->tpendSlot,
            g->rec, g->nsamples, g->vox, g->diff, g->spec, g->slotCap, g->voxCap, g->ntiles, g->st);
        CK(cudaGetLastError());
    }
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

static DevMap dev_map(DNgpuVolume* g)
{
    DevMap m;
    m.sx = g->sx; m.sy = g->sy; m.sz = g->sz;
    m.tword = g->tword; m.tbits = g->tbits; m.treq = g->treq; m.ttouch = g->ttouch; m.tvis = g->tvis;
    m.rec = g->rec; m.vox = g->vox; m.diff = g->diff; m.spec = g->spec;
    return m;
}

extern "C" int dn_cuda_light(DNgpuVolume* g, const dn_light_params* p, const dn_material* materials)
{
    if (!g || !p || !materials) return set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->K < 1 || p->K > 64) return set_err(DN_CUDA_ERR_ARG, "K = %u", p->K);
    CK(cudaSetDevice(g->device));
    CK(cudaMemsetAsync(&g->st->w[ST_WORK], 0, 4, g->stream));
    if (g_lightKernel == 0) {
        // one voxel per lane in lockstep phases (kept for comparison)
        static thread_local LightArgs* a = nullptr;
        if (!a) a = new LightArgs();
        a->m = dev_map(g);
        a->reqs = g->reqs; a->st = g->st; a->nsamples = g->nsamples; a->out = g->lightOut;
        a->p = *p;
        memcpy(a->mats, materials, sizeof(a->mats));
        int perSM = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light, 128, 0));
        if (perSM < 1) perSM = 1;
        COUNT_LAUNCH();
        k_light<<<g->numSMs * perSM, 128, 0, g->stream>>>(*a);
        CK(cudaGetLastError());
    } else {
        static thread_local StreamArgs* a = nullptr;
        if (!a) a = new StreamArgs();
        a->m = dev_map(g);
        a->reqs = g->reqs; a->workCounter = &g->st->w[ST_WORK]; a->nreqPtr = &g->st->w[ST_REQ];
        a->nsamples = g->nsamples; a->out = g->lightOut; a->stats = g->st->lstats;
        a->batch = g_streamBatch;
        a->p = *p;
        memcpy(a->mats, materials, sizeof(a->mats));
        int perSM = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light_stream, 128, 0));
        if (perSM < 1) perSM = 1;
        COUNT_LAUNCH();
        k_light_stream<<<g->numSMs * perSM, 128, 0, g->stream>>>(*a);
        CK(cudaGetLastError());
    }
    COUNT_LAUNCH();
    k_commit<<<g->numSMs * 4, 256, 0, g->stream>>>(dev_map(g), g->reqs, g->st, g->lightOut, g->diff, g->spec, g->nsamples);
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
// Limit: DN_NOALLOC_MAX_REQUESTS request groups (32 voxels each) per call; larger request lists are
// rejected with DN_CUDA_ERR_CAPACITY and a message naming both numbers.
// The array's device address is looked up once per device, on that device's first call (with the
// device current); that first call should come before any stream capture.  Every call shares the
// array and it keeps the previous call's contents: nothing in it needs to start at zero, because each
// call writes every slot it later reads.  Calls that overlap on the GPU (two volumes lit concurrently
// on different streams) race on the array.
#define DN_NOALLOC_MAX_REQUESTS 8192u   // 8192 groups x 32 lanes x 2 float4 = 8 MiB
static __device__ __align__(256) float4 g_noallocScratch[DN_NOALLOC_MAX_REQUESTS * 32u * 2u];

static std::mutex g_noallocMutex;
static float4* g_noallocAddr[64];      // device address of g_noallocScratch, per device ordinal

static int noalloc_scratch(int device, float4** out)
{
    if (device < 0 || device >= 64) return set_err(DN_CUDA_ERR_DEVICE, "device ordinal %d out of range", device);
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocAddr[device]) {
        float4* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noallocScratch);   // the device is current
        if (e != cudaSuccess || !ptr)
            return set_err(DN_CUDA_ERR_LAUNCH, "cudaGetSymbolAddress of the fixed lighting scratch: %s", cudaGetErrorString(e));
        g_noallocAddr[device] = ptr;
    }
    *out = g_noallocAddr[device];
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_light_noalloc(DNgpuVolume* g, const dn_light_params* p, const dn_material* materials)
{
    if (!g || !p || !materials) return set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->K < 1 || p->K > 64) return set_err(DN_CUDA_ERR_ARG, "K = %u", p->K);
    CK(cudaSetDevice(g->device));
    float4* scratch = nullptr;
    int rc = noalloc_scratch(g->device, &scratch);
    if (rc) return rc;
    // the request count exists only on the device: read it into the volume's pinned state block
    CK(cudaMemcpyAsync(&g->hst->w[ST_REQ], &g->st->w[ST_REQ], sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    const uint32_t nreq = g->hst->w[ST_REQ];
    if (nreq > DN_NOALLOC_MAX_REQUESTS)
        return set_err(DN_CUDA_ERR_CAPACITY,
                       "dn_cuda_light_noalloc: %u lighting request groups exceed the fixed scratch of %u groups "
                       "(%u voxels); use dn_cuda_light for this map", nreq, DN_NOALLOC_MAX_REQUESTS,
                       DN_NOALLOC_MAX_REQUESTS * 32u);
    CK(cudaMemsetAsync(&g->st->w[ST_WORK], 0, 4, g->stream));
    StreamArgs a;                       // launch arguments on the stack: no host allocation either
    a.m = dev_map(g);
    a.reqs = g->reqs; a.workCounter = &g->st->w[ST_WORK]; a.nreqPtr = &g->st->w[ST_REQ];
    a.nsamples = g->nsamples; a.out = scratch; a.stats = g->st->lstats;
    a.batch = g_streamBatch;
    a.p = *p;
    memcpy(a.mats, materials, sizeof(a.mats));
    int perSM = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_light_stream, 128, 0));
    if (perSM < 1) perSM = 1;
    COUNT_LAUNCH();
    k_light_stream<<<g->numSMs * perSM, 128, 0, g->stream>>>(a);
    CK(cudaGetLastError());
    COUNT_LAUNCH();
    k_commit<<<g->numSMs * 4, 256, 0, g->stream>>>(dev_map(g), g->reqs, g->st, scratch, g->diff, g->spec, g->nsamples);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

static int launch_draw(DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials, float4* color,
                       uint32_t* hit, uint8_t* face)
{
    static thread_local DrawArgs* a = nullptr;
    if (!a) a = new DrawArgs();
    a->m = dev_map(g);
    a->p = *p;
    a->color = color; a->hit = hit; a->face = face; a->stats = g->st->stats;
    memcpy(a->mats, materials, sizeof(a->mats));
    dim3 block(8, 32);
    dim3 grid((p->width + 7) / 8, (p->height + 31) / 32);
    COUNT_LAUNCH();
    k_draw<<<grid, block, 0, g->stream>>>(*a);
    CK(cudaGetLastError());
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_draw(DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials, float* colorOut,
                            uint32_t* hitOut, uint8_t* faceOut)
{
    if (!g || !p || !materials || !colorOut) return set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->width == 0 || p->height == 0) return set_err(DN_CUDA_ERR_ARG, "empty image");
    CK(cudaSetDevice(g->device));
    return launch_draw(g, p, materials, (float4*)colorOut, hitOut, faceOut);
}

extern "C" int dn_cuda_draw_host(DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials,
                                 float* colorOut, uint32_t* hitOut, uint8_t* faceOut)
{
    if (!g || !p || !materials || !colorOut) return set_err(DN_CUDA_ERR_ARG, "null argument");
    if (p->width == 0 || p->height == 0) return set_err(DN_CUDA_ERR_ARG, "empty image");
    CK(cudaSetDevice(g->device));
    const size_t n = (size_t)p->width * p->height;
    if (n > g->dimgCap) {
        CK(cudaStreamSynchronize(g->stream));
        dfree(g->dimg); dfree(g->dhit); dfree(g->dface);
        int rc;
        if ((rc = dalloc(&g->dimg, n)) || (rc = dalloc(&g->dhit, n)) || (rc = dalloc(&g->dface, n))) { g->dimgCap = 0; return rc; }
        g->dimgCap = n;
    }
    int rc = launch_draw(g, p, materials, g->dimg, hitOut ? g->dhit : nullptr, faceOut ? g->dface : nullptr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(colorOut, g->dimg, n * 16, cudaMemcpyDeviceToHost, g->stream));
    if (hitOut) CK(cudaMemcpyAsync(hitOut, g->dhit, n * 4, cudaMemcpyDeviceToHost, g->stream));
    if (faceOut) CK(cudaMemcpyAsync(faceOut, g->dface, n, cudaMemcpyDeviceToHost, g->stream));
    return DN_CUDA_OK;
}

// ----------------------------------------------------------- introspection

extern "C" int dn_cuda_finish(DNgpuVolume* g, uint64_t* numRequests)
{
    if (!g) return set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    CK(cudaMemcpyAsync(g->hst, g->st, sizeof(DevState), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    if (numRequests) *numRequests = g->hst->w[ST_REQ];
    if (g->hst->w[ST_ERR]) {
        uint32_t e = g->hst->w[ST_ERR];
        cudaMemsetAsync(&g->st->w[ST_ERR], 0, 4, g->stream);
        return set_err(DN_CUDA_ERR_KERNEL, "kernel error flags 0x%x", e);
    }
    return DN_CUDA_OK;
}

extern "C" int dn_cuda_stats_kind(DNgpuVolume* g, int kind, dn_stats* out)
{
    if (!g || !out || kind < 0 || kind > 2) return set_err(DN_CUDA_ERR_ARG, "bad argument");
    int rc = dn_cuda_finish(g, nullptr);
    if (rc && rc != DN_CUDA_ERR_KERNEL) return rc;
    unsigned long long s[8];
    for (int k = 0; k < 8; k++)
        s[k] = (kind != 2 ? g->hst->stats[k] : 0ull) + (kind != 1 ? g->hst->lstats[k] : 0ull);
    out->rays = s[S_RAYS]; out->primary = s[S_PRIMARY]; out->outerSteps = s[S_OUTER];
    out->chunksEntered = s[S_ENTERED]; out->innerSteps = s[S_INNER]; out->hits = s[S_HITS]; out->litVoxels = s[S_LIT];
    return rc;
}

extern "C" int dn_cuda_stats(DNgpuVolume* g, dn_stats* out) { return dn_cuda_stats_kind(g, 0, out); }

extern "C" int dn_cuda_reset_stats(DNgpuVolume* g)
{
    if (!g) return set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    CK(cudaMemsetAsync(g->st->stats, 0, sizeof(g->st->stats) + sizeof(g->st->lstats), g->stream));
    return DN_CUDA_OK;
}

extern "C" void* dn_cuda_stream(DNgpuVolume* g) { return g ? (void*)g->stream : nullptr; }

extern "C" int dn_cuda_export_tiles(DNgpuVolume* g, uint8_t* state, uint8_t* vis, uint32_t* lastUsed, uint32_t* samples)
{
    if (!g) return set_err(DN_CUDA_ERR_ARG, "null volume");
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    const uint64_t n = g->ntiles;
    uint32_t* tw = (uint32_t*)malloc(n * 4);
    uint8_t* rq = (uint8_t*)malloc(n);
    uint32_t* ns = (uint32_t*)malloc((size_t)g->slotCap * 4);
    if (!tw || !rq || !ns) { free(tw); free(rq); free(ns); return set_err(DN_CUDA_ERR_NOMEM, "host"); }
    cudaError_t e = cudaMemcpy(tw, g->tword, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rq, g->treq, n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && samples) e = cudaMemcpy(ns, g->nsamples, (size_t)g->slotCap * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && vis) e = cudaMemcpy(vis, g->tvis, n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && lastUsed) e = cudaMemcpy(lastUsed, g->tlast, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(tw); free(rq); free(ns); return set_err(DN_CUDA_ERR_LAUNCH, "copy: %s", cudaGetErrorString(e)); }
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
    if (!g || !count) return set_err(DN_CUDA_ERR_ARG, "null argument");
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
    if (!g || !count) return set_err(DN_CUDA_ERR_ARG, "null argument");
    CK(cudaSetDevice(g->device));
    CK(cudaStreamSynchronize(g->stream));
    const uint64_t n = g->ntiles;
    uint32_t* tw = (uint32_t*)malloc(n * 4);
    ChunkRec* rec = (ChunkRec*)malloc((size_t)g->slotCap * sizeof(ChunkRec));
    if (!tw || !rec) { free(tw); free(rec); return set_err(DN_CUDA_ERR_NOMEM, "host"); }
    cudaError_t e = cudaMemcpy(tw, g->tword, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rec, g->rec, (size_t)g->slotCap * sizeof(ChunkRec), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(tw); free(rec); return set_err(DN_CUDA_ERR_LAUNCH, "copy: %s", cudaGetErrorString(e)); }
    uint64_t rows = 0;
    for (uint64_t t = 0; t < n; t++)
        if ((tw[t] >> 30) == 2u) rows += rec[tw[t] & SLOT_MASK].nvox;
    *count = rows;
    if (!index || !diff || !spec) { free(tw); free(rec); return DN_CUDA_OK; }
    float4* hd = (float4*)malloc((size_t)g->voxCap * 16);
    float4* hs = (float4*)malloc((size_t)g->voxCap * 16);
    if (!hd || !hs) { free(tw); free(rec); free(hd); free(hs); return set_err(DN_CUDA_ERR_NOMEM, "host"); }
    e = cudaMemcpy(hd, g->diff, (size_t)g->voxCap * 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hs, g->spec, (size_t)g->voxCap * 16, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { free(tw); free(rec); free(hd); free(hs); return set_err(DN_CUDA_ERR_LAUNCH, "copy: %s", cudaGetErrorString(e)); }
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

extern "C" int dn_cuda_malloc(void** p, size_t bytes) { CK(cudaMalloc(p, bytes ? bytes : 1)); return DN_CUDA_OK; }
extern "C" int dn_cuda_free(void* p) { if (p) CK(cudaFree(p)); return DN_CUDA_OK; }
extern "C" int dn_cuda_malloc_host(void** p, size_t bytes) { CK(cudaMallocHost(p, bytes ? bytes : 1)); return DN_CUDA_OK; }
extern "C" int dn_cuda_free_host(void* p) { if (p) CK(cudaFreeHost(p)); return DN_CUDA_OK; }
extern "C" int dn_cuda_memcpy_d2h(void* dst, const void* src, size_t bytes) { CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost)); return DN_CUDA_OK; }
extern "C" int dn_cuda_memcpy_h2d(void* dst, const void* src, size_t bytes) { CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice)); return DN_CUDA_OK; }
extern "C" int dn_cuda_event_create(void** ev) { CK(cudaEventCreate((cudaEvent_t*)ev)); return DN_CUDA_OK; }
extern "C" int dn_cuda_event_destroy(void* ev) { CK(cudaEventDestroy((cudaEvent_t)ev)); return DN_CUDA_OK; }
extern "C" int dn_cuda_event_record(void* ev, void* stream) { CK(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream)); return DN_CUDA_OK; }
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
    return "k_draw;k_light;k_commit;k_sync_stage;k_compact;k_clamp_requests;k_flush";
}
