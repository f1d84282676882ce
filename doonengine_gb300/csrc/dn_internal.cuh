/*
 * dn_internal.cuh -- what the single-map entry points (dn_cuda.cu) and the
 * batched ones (dn_batch.cu) share: the per-map device state, error and
 * launch bookkeeping, and the per-pixel / per-tile / per-lane kernel bodies
 * that both the one-map kernels and the many-map kernels run.
 */
#pragma once
#include "dn_cuda.h"
#include "dn_device.cuh"
#include <cuda_runtime.h>
#include <stdint.h>

// ------------------------------------------------------------------ errors

int dn_set_err(int code, const char* fmt, ...);

#define CK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return dn_set_err(e_ == cudaErrorMemoryAllocation ? DN_CUDA_ERR_NOMEM : DN_CUDA_ERR_LAUNCH, \
                              "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// ------------------------------------------------------------------ state

// ST_LIMITED: the request count a dn_cuda_light_noalloc launch lights (its own count, or 0 when the
// list exceeds the fixed scratch; k_noalloc_guard writes it)
enum { ST_REQ = 0, ST_WORK = 1, ST_ERR = 2, ST_LIMITED = 3 };
// error flag bits of ST_ERR (reported by dn_cuda_finish / dn_cuda_batch_finish)
enum : uint32_t { ERRF_TILE = 1u, ERRF_RECORD = 2u, ERRF_REQUESTS = 4u, ERRF_NOALLOC_CAPACITY = 0x100u };
enum { S_RAYS = 0, S_PRIMARY, S_OUTER, S_ENTERED, S_INNER, S_HITS, S_LIT, S_DEGEN, S_COUNT };

struct DevState {
    uint32_t w[4];                      // nreq, work counter, error flags, noalloc request count
    unsigned long long stats[8];        // draw kernels
    unsigned long long lstats[8];       // lighting kernels
};

struct DNgpuBatch;
namespace dn { struct LightTables; }   // dn_light_stream.cuh

struct DNgpuVolume {
    int device;
    cudaStream_t stream;                // the batch's stream while the volume belongs to a batch
    cudaStream_t ownStream;
    DNgpuBatch* batch;
    uint64_t gen;                       // unique per allocation state (dn_new_generation)
    uint32_t sx, sy, sz;
    uint64_t ntiles;
    uint32_t* tword; uint8_t* treq; uint8_t* tvis; uint8_t* ttouch;
    uint32_t* tbits;                    // 2 bits per tile: 0 absent, 1 unloaded, 2 loaded (16 tiles per word)
    uint32_t* tlast; uint32_t* tpend; uint32_t* tpendSlot;
    dn::ChunkRec* rec; uint32_t* nsamples; uint32_t slotCap;
    uint2* vox; float4* diff; float4* spec; uint64_t voxCap;
    uint32_t* reqs; float4* lightOut; uint64_t reqCap;
    DevState* st;
    dn::LightTables* dtab;              // materials and shadow directions of the last lighting launch (k_light_packet)
    // pinned staging for sync uploads and small readbacks
    // two pinned upload buffers: a sync takes one whose last upload is done, so the host does not wait for
    // the previous sync's upload while that sync's work is still queued (a tick in flight)
    unsigned char* hstage[2]; size_t hstageCap[2];
    unsigned char* dstage; size_t dstageCap;
    cudaEvent_t stageFree[2];   // after each buffer's last upload
    int stageCur;               // the buffer of the last upload
    cudaEvent_t copyDone;       // eviction / restore: the volume's queued work, then its last copy on the copy stream
    int restorePending;         // restored by dn_cuda_map_restore_async: the volume's stream has not waited yet
    DevState* hst;                      // pinned copy of DevState
    // device staging for host-memory draws
    float4* dimg; uint32_t* dhit; uint8_t* dface; size_t dimgCap;
    int numSMs;
    // eviction: every persistent device array copied into slabs of the process-wide pinned host pool
    // (evicted: the slabs' indices, null while resident), device arrays freed
    uint32_t* evicted; uint32_t evictedSlabs;
    // arrays allocated from the device's stream-ordered pool (bit per array, vol_array_bit): freed with
    // cudaFreeAsync on the volume's stream instead of cudaFree (which waits for the whole device)
    uint32_t poolMask;
};



#ifndef DN_DRAW_MIN_BLOCKS
// resident 256-thread draw blocks per SM the register allocation must allow: 3 (80 registers, a few spills)
// against 2 at 96 registers; measured +0.9 % on the batched workload and +1.2 % on the streaming one, where
// the draw is a quarter of the frame (4: 64 registers, more spills, no gain)
#define DN_DRAW_MIN_BLOCKS 3
#endif

extern int g_device;
extern int g_numSMs;
extern unsigned long long g_launches;   // kernels launched by this library (all threads)
extern int g_lightKernel;               // 1 per-lane ray streams, 2 warp packets (default)
extern uint32_t g_streamBatch;          // lanes that wait before per-segment work runs (1..32), ray streams
extern uint32_t g_packetBatch;          // the same threshold for the packet kernel's ray pools
#define COUNT_LAUNCH() __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED)
extern unsigned long long g_allocs;     // device and pinned allocations made by this library (all threads)
#define COUNT_ALLOC() __atomic_fetch_add(&g_allocs, 1ull, __ATOMIC_RELAXED)

template <class T> static int dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    COUNT_ALLOC();
    CK(cudaMalloc((void**)p, count * sizeof(T)));
    return DN_CUDA_OK;
}
template <class T> static void dfree(T*& p) { if (p) cudaFree(p); p = nullptr; }

// the bit of one of the volume's device arrays (its field address) in poolMask; 0 for other pointers
uint32_t vol_array_bit(DNgpuVolume* g, const void* field);
extern bool g_asyncAlloc;               // the device supports stream-ordered allocation (cudaMallocAsync)

// frees one of the volume's device arrays: stream-ordered on stream s (the volume's stream by default) when
// it came from the pool
template <class T> static void vfree(DNgpuVolume* g, T*& p, cudaStream_t s = nullptr)
{
    if (!p) return;
    const uint32_t bit = vol_array_bit(g, &p);
    if (bit && (g->poolMask & bit)) cudaFreeAsync(p, s ? s : g->stream);
    else cudaFree(p);
    g->poolMask &= ~bit;
    p = nullptr;
}
// allocates one of the volume's device arrays from the stream-ordered pool, ordered on stream s (the
// volume's stream by default: work issued afterwards on that stream may use it)
template <class T> static int valloc(DNgpuVolume* g, T*& p, size_t count, cudaStream_t s = nullptr)
{
    p = nullptr;
    if (count == 0) count = 1;
    const uint32_t bit = vol_array_bit(g, &p);
    COUNT_ALLOC();
    if (g_asyncAlloc && bit) {
        CK(cudaMallocAsync((void**)&p, count * sizeof(T), s ? s : g->stream));
        g->poolMask |= bit;
    } else {
        CK(cudaMalloc((void**)&p, count * sizeof(T)));
    }
    return DN_CUDA_OK;
}

// An evicted map cannot be used.  A map restored by dn_cuda_map_restore_async gets its stream's wait for the
// restore copies here, so that the work an entry point queues next sees its arrays.
static inline bool map_evicted(DNgpuVolume* g)
{
    if (g->evicted) return true;
    if (g->restorePending) {
        cudaStreamWaitEvent(g->stream, g->copyDone, 0);
        g->restorePending = 0;
    }
    return false;
}

static inline dn::DevMap dev_map(const DNgpuVolume* g)
{
    dn::DevMap m;
    m.sx = g->sx; m.sy = g->sy; m.sz = g->sz;
    const uint64_t cap = 256ull * ((uint64_t)g->sx + g->sy + g->sz) + 4096ull;   // step_cap (dn_device.cuh)
    m.stepCap = cap > (1ull << 23) ? (1u << 23) : (uint32_t)cap;
    m.tword = g->tword; m.tbits = g->tbits; m.treq = g->treq; m.ttouch = g->ttouch; m.tvis = g->tvis;
    m.rec = g->rec; m.vox = g->vox; m.diff = g->diff; m.spec = g->spec;
    m.degen = nullptr;                   // set by the launch: the draw's or the lighting's counter
    return m;
}

// the staging half of a sync (host ops -> records and voxels); compaction follows separately
int dn_stage_ops(DNgpuVolume* g, const dn_tile_op* ops, uint32_t nops, const dn_chunk_record* records,
                 uint32_t nrecords, const uint32_t* voxelWords, uint64_t nvoxels);
// grows the device staging of host-memory draws to n pixels
int dn_reserve_image_staging(DNgpuVolume* g, size_t n);
// checks a draw's raster composition arguments (host side, before any launch)
int dn_check_raster(const dn_draw_params* p);
// gives g a new process-wide unique generation (after any device array of g is reallocated)
void dn_new_generation(DNgpuVolume* g);

// ------------------------------------------------------------ counters

__device__ __forceinline__ uint32_t lane_id()
{
    uint32_t l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

__device__ __forceinline__ void flush_counters(unsigned long long* stats, const dn::Counters& c, uint32_t primary, uint32_t lit)
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

// ------------------------------------------------- opaque chunks of a lighting launch

// The lighting step (seg_step) reads the 2-bit tile map; before each lighting launch a loaded chunk whose
// voxels all use materials that are opaque under the launch's materials is marked 3 instead of 2.  A ray
// that reaches an occupied voxel of such a chunk ends there without reading the voxel's word and material
// (its pool index is formed when the segment is shaded).  The next sync rewrites the map with 0 / 1 / 2.

// opq[8] (shared memory): bit m set when material m is opaque (opacity exactly 1, voxelShared.comp:360)
__device__ __forceinline__ void opaque_materials(const dn::Material* mats, uint32_t* opq)
{
    if (threadIdx.x < 8) opq[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t m = threadIdx.x; m < 256; m += blockDim.x)
        if (mats[m].opacity == 1.0f) atomicOr(&opq[m >> 5], 1u << (m & 31u));
    __syncthreads();
}

// word wi of the map's 2-bit tile map (16 tiles): every loaded tile to 3 (all materials opaque) or 2
__device__ __forceinline__ void mark_opaque_word(uint32_t* tbits, const uint32_t* tword, const dn::ChunkRec* rec,
                                                 uint64_t wi, const uint32_t* opq)
{
    const uint32_t w = tbits[wi];
    uint32_t out = w;
    for (uint32_t k = 0; k < 16; k++) {
        if (((w >> (2 * k)) & 2u) == 0u) continue;
        const uint32_t slot = __ldg(&tword[wi * 16 + k]) & dn::SLOT_MASK;
        const uint32_t* ms = rec[slot].matSet;
        uint32_t other = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) other |= __ldg(&ms[j]) & ~opq[j];
        out = (out & ~(3u << (2 * k))) | ((other ? 2u : 3u) << (2 * k));
    }
    if (out != w) tbits[wi] = out;
}

// ------------------------------------------------------------------ draw

// one image of one map
struct DrawMap {
    dn::DevMap m;
    dn_draw_params p;
    float4* color;
    uint32_t* hit;
    uint8_t* face;
    unsigned long long* stats;
};

struct DrawArgs {
    DrawMap d;
    dn::Material mats[256];
};

// Texel index of floor coordinate f under GL_REPEAT wrapping on a texture n texels wide.
__device__ __forceinline__ uint32_t repeat_texel(float f, uint32_t n)
{
    const int k = (int)f % (int)n;
    return (uint32_t)(k < 0 ? k + (int)n : k);
}

// GL_LINEAR sample with GL_REPEAT wrapping at texture coordinate (s, t), the filtering of the reference's
// raster textures (main.c:313-322; wrap left at its default).  The steps are the OpenGL 4.3 formula
// (section 8.14.2): u = s*w - 1/2, i0 = wrap(floor(u)), i1 = wrap(floor(u) + 1), alpha = u - floor(u),
// the same along t, then (1-a)(1-b) T00 + a(1-b) T10 + (1-a)b T01 + ab T11 summed in that order.  C floats
// per texel; the first N are returned.
template <int C, int N>
__device__ __forceinline__ void raster_sample(const float* tex, uint32_t w, uint32_t h, float s, float t, float* out)
{
    const float u = s * (float)w - 0.5f, v = t * (float)h - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const uint32_t i0 = repeat_texel(fu, w), j0 = repeat_texel(fv, h);
    const uint32_t i1 = i0 + 1u == w ? 0u : i0 + 1u, j1 = j0 + 1u == h ? 0u : j0 + 1u;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    const float* t00 = tex + ((size_t)j0 * w + i0) * C;
    const float* t10 = tex + ((size_t)j0 * w + i1) * C;
    const float* t01 = tex + ((size_t)j1 * w + i0) * C;
    const float* t11 = tex + ((size_t)j1 * w + i1) * C;
#pragma unroll
    for (int k = 0; k < N; k++)
        out[k] = w00 * __ldg(t00 + k) + w10 * __ldg(t10 + k) + w01 * __ldg(t01 + k) + w11 * __ldg(t11 + k);
}

// One primary ray (voxelDraw.comp:24-147): pixel (x, y) of the image described by a; smat holds the map's
// materials.  Returns 1 when a primary ray was traced.
__device__ __forceinline__ uint32_t draw_pixel(const DrawMap& a, const dn::Material* smat, uint32_t x, uint32_t y,
                                               dn::Counters& cnt)
{
    using namespace dn;
    const dn_draw_params& p = a.p;
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
            // raster depth as a distance from the camera (voxelDraw.comp:86-101); negative: not tested
            float maxDepth = -1.0f;
            float texS = 0.0f, texT = 0.0f;
            if (p.compose) {
                texS = (float)x / (float)p.rasterColorW;
                texT = (float)y / (float)p.rasterColorH;
                float d;
                raster_sample<1, 1>(p.rasterDepth, p.rasterDepthW, p.rasterDepthH, texS, texT, &d);
                maxDepth = d * 2.0f - 1.0f;
                if (maxDepth < 1.0f) {
                    const float (*P)[4] = p.invProj;
                    float vs[4];
#pragma unroll
                    for (int r = 0; r < 4; r++) vs[r] = P[0][r] * sx + P[1][r] * sy + P[2][r] * maxDepth + P[3][r] * 1.0f;
                    const float wv = vs[3];
                    const f3 vsp = mk(vs[0] / wv, vs[1] / wv, vs[2] / wv);
                    maxDepth = sqrtf(dot(vsp, vsp));
                } else {
                    maxDepth = -1.0f;
                }
            }
            // background_color (voxelDraw.comp:24-30): the sky, or the raster colour where a depth is tested
            auto background = [&](f3 dir) -> f3 {
                if (maxDepth < 0.0f) {
                    const f3 s = sky_color(mk(p.skyBot[0], p.skyBot[1], p.skyBot[2]), mk(p.skyTop[0], p.skyTop[1], p.skyTop[2]), dir);
                    return mk(powf(s.x, 2.2f), powf(s.y, 2.2f), powf(s.z, 2.2f));
                }
                float rc[3];
                raster_sample<4, 3>(p.rasterColor, p.rasterColorW, p.rasterColorH, texS, texT, rc);
                return mk(rc[0], rc[1], rc[2]);
            };
            const f3 mapMax = mk((float)a.m.sx, (float)a.m.sy, (float)a.m.sz);
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
                fc = background(rayDir);
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
                    if (maxDepth > 0.0f && depth > maxDepth) {
                        // the rasterised scene is in front of the voxel (voxelDraw.comp:127-131): the pixel shows
                        // it, so no voxel is reported as hit
                        fc = add(muls(background(rayDir), cmul), cadd);
                        depth = maxDepth;
                    } else {
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
                    }
                } else {
                    fc = add(muls(background(rayDir), cmul), cadd);
                    depth = maxDepth;
                }
            }
            out = make_float4(powf(fc.x, 0.4545f), powf(fc.y, 0.4545f), powf(fc.z, 0.4545f), depth);
        }
        a.color[pix] = out;
        if (a.hit) a.hit[pix] = hitIdx;
        if (a.face) a.face[pix] = face;
    }
    cnt = c.c;
    return primary;
}

// -------------------------------------------------------------- sync

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
    const dn::ChunkRec* rec;
    uint32_t* reqs; uint64_t reqCap;
    DevState* st;
    uint64_t ntiles;
    uint32_t op, split, frameNum;
};

// Tiles [base, base + blockDim.x) of one map: the per-tile loop of DN_sync_gpu (voxel.c:738-762) with the
// request rule of _DN_request_chunk_lighting (1463-1489) and the state machine of _DN_stream_to_gpu
// (1491-1536).  blockDim.x is a multiple of 32 and base a multiple of 32.
__device__ __forceinline__ void compact_tiles(const CompactArgs& a, uint64_t base)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t t = base + threadIdx.x;
    uint32_t groups = 0;
    uint32_t finalSt = 0;
    if (t < a.ntiles) {
        const uint32_t w = a.tword[t];
        const uint32_t st = w >> 30;
        finalSt = st;
        uint32_t slot = w & dn::SLOT_MASK;
        const uint32_t pend = a.tpend[t];
        const bool req = a.treq[t] != 0;
        uint32_t vis = a.tvis[t];
        uint32_t gflag = (st == 1u && req) ? 3u : st;
        // an earlier tile of this sync took the chunk's node (DN_RESIDENCY_LRU): it reaches its turn unloaded
        if (pend & DN_PEND_EVICTED) { gflag = 1u; vis = 0; slot = DN_SLOT_NONE; }
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
            // a load; with DN_RESIDENCY_LRU it can find no node and leave the chunk unloaded
            const bool hold = (pend & DN_PEND_HOLD) != 0;
            if (gflag == 3u && exists && (hold || newSlot != DN_SLOT_NONE)) { gflag = hold ? 1u : 2u; lu = 0; changed = true; }
            // a later tile of this sync took the chunk's node
            if (pend & DN_PEND_EVICT) { gflag = 1u; changed = true; }
            if (changed) vis = 0;
            slot = (exists && !(pend & (DN_PEND_EVICT | DN_PEND_EVICTED))) ? newSlot : DN_SLOT_NONE;
            a.treq[t] = (gflag == 3u) ? 1 : 0;
            finalSt = gflag == 3u ? 1u : gflag;
            a.tword[t] = (finalSt << 30) | (slot & dn::SLOT_MASK);
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
            else atomicOr(&a.st->w[ST_ERR], ERRF_REQUESTS);
        }
    }
}

// D1/D2: lane `lane` of request r of one map: copy its new lighting into the pool and count the sample
__device__ __forceinline__ void commit_lane(const dn::DevMap& m, const uint32_t* reqs, const float4* out, uint64_t i,
                                            uint32_t r, uint32_t lane, float4* diff, float4* spec, uint32_t* nsamples)
{
    const uint32_t word = reqs[r];
    const uint32_t tile = word >> 4, group = word & 15u;
    const uint32_t tw = m.tword[tile];
    if ((tw >> 30) != 2u) return;
    const uint32_t slot = tw & dn::SLOT_MASK;
    const dn::ChunkRec* rc = &m.rec[slot];
    const uint32_t vn = group * 32u + lane;
    if (vn >= rc->nvox) return;
    const uint32_t idx = rc->voxBase + vn;
    diff[idx] = out[i * 2u];
    spec[idx] = out[i * 2u + 1u];
    if (vn == 0) nsamples[slot] += 1u;
}
