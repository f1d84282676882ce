/*
 * dn_device.cuh -- device-side traversal and shading for sm_103a.
 *
 * The two-level chunk-skipping DDA (voxelShared.comp:300-475), the lighting
 * rays (voxelLighting.comp:65-288) and the primary-ray shading
 * (voxelDraw.comp:24-147), written for CUDA.  Every floating-point expression
 * keeps the reference's operation order and this file is compiled with
 * --fmad=false and IEEE division / square root, so a ray takes exactly the
 * same steps as on the host and hit voxels match bit for bit.
 *
 * Deterministic semantics (shared with the CPU oracle, numbered as there):
 *   D1 lighting reads last frame's committed lighting, new values are
 *      committed by a second kernel; D2 sample count snapshotted per launch;
 *   D3 FP32 lighting; D4 visible / requested / touched are per-tile bytes
 *      written with idempotent stores; D5 per-ray integer-hash RNG (or the
 *      reference's sin-fract with a deterministic sine); D6 bounded
 *      rejection sampling; D8 K fixed direct / specular rays; D9 emissive
 *      strength; D11 no FMA, IEEE div/sqrt, GLSL built-ins by their
 *      specification formulas; D13 transparency state fresh per ray job;
 *      D14 face code and global hit index.
 */
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace dn {

constexpr float EPS = 0.0001f;            // voxelShared.comp:7
constexpr float INV_CHUNK = 0.125f;       // voxelShared.comp:4
constexpr float HALF_INV_CHUNK = 0.0625f; // voxelShared.comp:5
constexpr float INV255 = 0.00392156862f;  // voxelShared.comp:249-253
constexpr uint32_t SLOT_MASK = 0x3FFFFFFFu;

struct f3 { float x, y, z; };
struct i3 { int32_t x, y, z; };

__device__ __forceinline__ f3 mk(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 mul(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 muls(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 adds(f3 a, float s) { return mk(a.x + s, a.y + s, a.z + s); }
__device__ __forceinline__ f3 divs(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// GLSL min/max: min(x, y) = y < x ? y : x; max(x, y) = x < y ? y : x
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gsign(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }
__device__ __forceinline__ f3 normalize(f3 v) { float l = sqrtf(dot(v, v)); return divs(v, l); }
__device__ __forceinline__ f3 vabs(f3 v) { return mk(fabsf(v.x), fabsf(v.y), fabsf(v.z)); }
__device__ __forceinline__ f3 vfloor(f3 v) { return mk(floorf(v.x), floorf(v.y), floorf(v.z)); }
__device__ __forceinline__ float min3(f3 v) { return gmin(gmin(v.x, v.y), v.z); }
__device__ __forceinline__ f3 reflect(f3 I, f3 N) { float t = 2.0f * dot(N, I); return sub(I, muls(N, t)); }
__device__ __forceinline__ f3 refract(f3 I, f3 N, float eta)
{
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    float s = eta * d + sqrtf(k);
    return sub(muls(I, eta), muls(N, s));
}
// float -> int32 with saturation, NaN -> 0
__device__ __forceinline__ int32_t f2i(float x)
{
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 0x7FFFFFFF;
    if (x < -2147483648.0f) return (int32_t)0x80000000;
    return (int32_t)x;
}

// ---------------------------------------------------------------- RNG (D5)

__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    // 32-bit integer finaliser ("lowbias32", C. Wellons' hash-prospector)
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ uint32_t rng_key(uint32_t seed, uint32_t mapId, uint32_t voxel)
{
    return hash32(seed ^ hash32(voxel ^ hash32(mapId + 0x632be5abu)));
}
__device__ __forceinline__ float hrand(uint32_t key, uint32_t stream, uint32_t idx)
{
    uint32_t h = hash32(key ^ hash32((stream << 28) ^ idx));
    return (float)(h >> 8) * (1.0f / 8388608.0f) - 1.0f;
}
// deterministic sine: Cody-Waite reduction by pi/2 and Taylor polynomials on [-pi/4, pi/4]
__device__ __forceinline__ float det_sin(float x)
{
    const float P1 = 1.5703125f, P2 = 4.837512969970703125e-4f, P3 = 7.549790126404332e-8f;
    float kf = floorf(x * 0.636619746685028076f + 0.5f);
    float r = ((x - kf * P1) - kf * P2) - kf * P3;
    float r2 = r * r;
    int32_t q = f2i(kf) & 3;
    float s = r + r * r2 * (-0.16666667163372040f + r2 * (0.0083333337679505f +
              r2 * (-0.00019841270113829523f + r2 * 2.7557318844628753e-06f)));
    float c = 1.0f + r2 * (-0.5f + r2 * (0.0416666679084301f + r2 * (-0.0013888889225199819f +
              r2 * (2.4801587642286904e-05f + r2 * -2.755731998149713e-07f))));
    return q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}
__device__ __forceinline__ float srand1(float s) { float v = det_sin(s) * 43758.5453f; return (v - floorf(v)) * 2.0f - 1.0f; }
static __device__ __noinline__ f3 sphere_sin(float seed)
{
    for (int t = 0; t < 64; t++) {
        float s = seed;
        seed = seed + 1.0f;
        f3 p = mk(srand1(s), srand1(s * 2.0f), srand1(s * 3.0f));
        if (dot(p, p) >= 1.0f) continue;
        return p;
    }
    return mk(0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ f3 sphere_hash(uint32_t key, uint32_t stream, uint32_t base)
{
    for (uint32_t t = 0; t < 64; t++) {
        uint32_t i = (base << 8) | (3u * t);
        f3 p = mk(hrand(key, stream, i), hrand(key, stream, i + 1u), hrand(key, stream, i + 2u));
        if (dot(p, p) >= 1.0f) continue;
        return p;
    }
    return mk(0.0f, 0.0f, 0.0f);
}

// ------------------------------------------------------------ map layout

// chunk record, 128 B: occupancy mask (bit x + 8*(y + 8*z)), partial counts, voxel count, position, pool base,
// and the set of materials its voxels use (bit m of matSet[m >> 5]; written when the chunk is staged)
struct __align__(128) ChunkRec {
    uint32_t mask[16];
    uint32_t partial[3];
    uint32_t nvox;
    int32_t pos[3];
    uint32_t voxBase;
    uint32_t matSet[8];
};

struct Material {             // 32 B, DNmaterial
    float pad0, pad1;
    uint32_t emissive;
    float opacity, refractIndex, specular;
    uint32_t reflectType, shininess;
};

struct Counters {             // per-thread traversal counters
    uint32_t rays, outer, entered, inner, hits;
};

struct DevMap {
    uint32_t sx, sy, sz;
    uint32_t stepCap;                    // D16: cells a traversal segment may visit (step_cap of the size)
    const uint32_t* __restrict__ tword;  // state << 30 | slot
    const uint32_t* __restrict__ tbits;  // 2 bits per tile: 0 absent, 1 unloaded, 2 loaded
    uint8_t* treq;
    uint8_t* ttouch;
    uint8_t* tvis;
    const ChunkRec* __restrict__ rec;
    const uint2* __restrict__ vox;       // normal word, linear albedo word
    const float4* __restrict__ diff;
    const float4* __restrict__ spec;
    unsigned long long* degen;           // D16: segments ended at once for a degenerate direction (counter)
};

struct Voxel { f3 normal; uint32_t material; f3 albedo; f3 spec; f3 diff; };
struct TState { uint32_t lastVoxID; float lastVoxRefract; };
struct HitInfo { uint32_t tile; i3 local; };

__device__ __forceinline__ bool in_chunk(i3 p) { return p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < 8 && p.y < 8 && p.z < 8; }
__device__ __forceinline__ bool in_map(const DevMap& m, i3 p)
{
    return p.x >= 0 && p.y >= 0 && p.z >= 0 && (uint32_t)p.x < m.sx && (uint32_t)p.y < m.sy && (uint32_t)p.z < m.sz;
}
__device__ __forceinline__ uint32_t map_index(const DevMap& m, i3 p)
{
    return (uint32_t)p.x + m.sx * ((uint32_t)p.y + m.sy * (uint32_t)p.z);
}

// rank of voxel li among the set bits (get_voxel_index, voxelShared.comp:150-169)
__device__ __forceinline__ uint32_t vox_rank(const ChunkRec* r, uint32_t li)
{
    uint32_t w = li >> 5;
    uint32_t n = (w > 3) ? __ldg(&r->partial[(w >> 2) - 1]) : 0u;
    for (uint32_t i = w & ~3u; i < w; i++) n += __popc(__ldg(&r->mask[i]));
    return n + __popc(__ldg(&r->mask[w]) & ((1u << (li & 31)) - 1u));
}

__device__ __forceinline__ void decompress(const DevMap& m, uint32_t idx, Voxel& v)
{
    // decompress_voxel, voxelShared.comp:236-256, FP32 lighting
    uint2 w = __ldg(&m.vox[idx]);
    v.normal = mk(((float)((w.x >> 16) & 0xFF) * INV255 - 0.5f) * 2.0f,
                  ((float)((w.x >> 8) & 0xFF) * INV255 - 0.5f) * 2.0f,
                  ((float)(w.x & 0xFF) * INV255 - 0.5f) * 2.0f);
    v.material = w.x >> 24;
    v.albedo = mk((float)((w.y >> 24) & 0xFF) * INV255, (float)((w.y >> 16) & 0xFF) * INV255,
                  (float)((w.y >> 8) & 0xFF) * INV255);
    float4 d = __ldg(&m.diff[idx]);
    float4 s = __ldg(&m.spec[idx]);
    v.diff = mk(d.x, d.y, d.z);
    v.spec = mk(s.x, s.y, s.z);
}

// init_DDA, voxelShared.comp:300-306
__device__ __forceinline__ void init_dda(f3 dir, f3 inv, f3 p, i3& pos, f3& delta, i3& step, f3& side)
{
    f3 fl = vfloor(p);
    pos.x = f2i(fl.x); pos.y = f2i(fl.y); pos.z = f2i(fl.z);
    delta = vabs(inv);
    f3 s = mk(gsign(dir.x), gsign(dir.y), gsign(dir.z));
    step.x = f2i(s.x); step.y = f2i(s.y); step.z = f2i(s.z);
    side.x = (s.x * ((float)pos.x - p.x) + s.x * 0.5f + 0.5f) * delta.x;
    side.y = (s.y * ((float)pos.y - p.y) + s.y * 0.5f + 0.5f) * delta.y;
    side.z = (s.z * ((float)pos.z - p.z) + s.z * 0.5f + 0.5f) * delta.z;
}

// iterate_DDA, voxelShared.comp:309-317 (<= steps; ties step several axes), for finite, non-negative side
// distances (every caller has a finite direction, D16, and the side distances start at +0 or above):
// fminf then gives GLSL min's value, and adding delta only on the stepped axes gives exactly
// side + (mask ? 1 : 0) * delta.  Returns min3 of the side distances before the step, the only use the
// reference makes of lastSideDist, and the stepped axes in nmask (bits 0-2): settle_normal forms
// iterate_DDA's normal output from them where it is read (a hit, a refraction, the end of the traversal)
// instead of on every step.  (Measured on the draw against the literal form, bit-identical: streaming
// edits +2.5-3.5 %, batched workload +1.2 %, 148 bytes of spills down to 48.)
__device__ __forceinline__ float iter_dda_min(f3 delta, i3 step, f3& side, i3& pos, uint32_t& nmask)
{
    const float gyz = fminf(side.y, side.z), gzx = fminf(side.z, side.x), gxy = fminf(side.x, side.y);
    const float lastMin = fminf(gxy, side.z);
    const bool mx = side.x <= gyz, my = side.y <= gzx, mz = side.z <= gxy;
    if (mx) side.x = side.x + delta.x;
    if (my) side.y = side.y + delta.y;
    if (mz) side.z = side.z + delta.z;
    pos.x += (int32_t)mx * step.x; pos.y += (int32_t)my * step.y; pos.z += (int32_t)mz * step.z;
    nmask = (mx ? 1u : 0u) | (my ? 2u : 0u) | (mz ? 4u : 0u);
    return lastMin;
}
// iterate_DDA's normal output of the last step, formed from its stepped axes when it is read
__device__ __forceinline__ void settle_normal(f3& normal, uint32_t& nmask, i3 step)
{
    if (nmask) {
        normal.x = ((nmask & 1u) ? 1.0f : 0.0f) * (float)(-step.x);
        normal.y = ((nmask & 2u) ? 1.0f : 0.0f) * (float)(-step.y);
        normal.z = ((nmask & 4u) ? 1.0f : 0.0f) * (float)(-step.z);
        nmask = 0;
    }
}

struct RayCtx {
    const DevMap* m;
    const Material* mats;     // shared-memory copy
    f3 sunStrength;
    float emissive;
    bool refraction;
    f3 orgRayPos;
    Counters c;
    uint32_t segSteps;        // cells visited by the current step_map call (D16)
    bool capped;
};

// D16: a traversal segment whose direction has a zero or NaN component -- its reciprocal is then infinite
// or NaN -- traverses nothing and ends at once as a miss (counted in DevMap::degen).  The reference's side
// distances become NaN after one step of such a ray (0 * inf), after which no axis may be stepped again and
// its loops (voxelShared.comp:339, 435) never end; reflect() without an added EPSILON
// (voxelLighting.comp:132, 163) produces such directions.  With a finite direction every DDA step advances
// one axis monotonically (at most sx+sy+sz chunk cells and 24 voxel cells per chunk entered); the cell cap
// below ends only repeated refraction inside transparent voxels (the draw).
__device__ __forceinline__ bool finite_dir(f3 inv) { return isfinite(inv.x) && isfinite(inv.y) && isfinite(inv.z); }
__device__ __forceinline__ void count_degenerate(const DevMap& m) { if (m.degen) atomicAdd(m.degen, 1ull); }
__device__ __forceinline__ uint32_t step_cap(uint32_t sx, uint32_t sy, uint32_t sz)
{
    const uint64_t c = 256ull * ((uint64_t)sx + sy + sz) + 4096ull;
    return c > (1ull << 23) ? (1u << 23) : (uint32_t)c;
}

// step_chunk, voxelShared.comp:328-418
static __device__ __forceinline__ bool step_chunk(RayCtx& c, TState& ts, i3 mapPos, uint32_t slot, uint32_t tile,
                                        f3& rayDir, f3& inv, f3& rayPos, bool ignoreFirst, float maxDepth,
                                        f3& hitNormal, Voxel& vox, f3& colorAdd, float& colorMult,
                                        bool& refracted, HitInfo& hi)
{
    const DevMap& m = *c.m;
    const ChunkRec* r = &m.rec[slot];
    const uint32_t base = __ldg(&r->voxBase);
    refracted = false;
    i3 pos, step; f3 delta, side;
    float lastMin = 0.0f;   // min3(lastSideDist)
    uint32_t nmask = 0;       // stepped axes of the last DDA step whose normal is not yet formed
    init_dda(rayDir, inv, rayPos, pos, delta, step, side);
    const uint32_t cap = step_cap(m.sx, m.sy, m.sz);
    while (in_chunk(pos)) {
        if (c.segSteps >= cap) { settle_normal(hitNormal, nmask, step); c.capped = true; return false; }
        c.segSteps++;
        c.c.inner++;
        uint32_t li = (uint32_t)(pos.x + 8 * (pos.y + 8 * pos.z));
        bool exists = (__ldg(&r->mask[li >> 5]) >> (li & 31)) & 1u;
        if (exists && !ignoreFirst) {
            uint32_t idx = base + vox_rank(r, li);
            c.c.hits++;
            decompress(m, idx, vox);
            const Material& mat = c.mats[vox.material];
            uint2 w = __ldg(&m.vox[idx]);
            uint32_t thisID = (w.y & 0xFFFFFF00u) | (w.x >> 24);
            if (mat.opacity == 1.0f) {
                float t = lastMin + EPS;
                rayPos = add(rayPos, muls(rayDir, t));
                hi.tile = tile; hi.local = pos;
                settle_normal(hitNormal, nmask, step);
                return true;
            } else if (ts.lastVoxID != thisID) {
                f3 cur = add(rayPos, muls(rayDir, lastMin));
                cur = add(mk((float)mapPos.x, (float)mapPos.y, (float)mapPos.z), muls(cur, INV_CHUNK));
                f3 to = sub(cur, c.orgRayPos);
                if (maxDepth < 0.0f || dot(to, to) < maxDepth * maxDepth) {
                    float k = colorMult * mat.opacity;
                    colorAdd.x = colorAdd.x + k * vox.albedo.x * c.sunStrength.x;
                    colorAdd.y = colorAdd.y + k * vox.albedo.y * c.sunStrength.y;
                    colorAdd.z = colorAdd.z + k * vox.albedo.z * c.sunStrength.z;
                    colorMult = colorMult * (1.0f - mat.opacity);
                }
                float rd = lastMin;
                if (c.refraction && rd > 0.0f) {
                    refracted = true;
                    rayPos = add(rayPos, muls(rayDir, rd + EPS));
                    settle_normal(hitNormal, nmask, step);
                    f3 n = (dot(vox.normal, rayDir) < 0.0f) ? normalize(vox.normal) : hitNormal;
                    rayDir = refract(rayDir, n, ts.lastVoxRefract / mat.refractIndex);
                    inv = mk(1.0f / rayDir.x, 1.0f / rayDir.y, 1.0f / rayDir.z);
                    if (!finite_dir(inv)) { count_degenerate(m); c.capped = true; return false; }
                    init_dda(rayDir, inv, rayPos, pos, delta, step, side);
                    lastMin = 0.0f;
                }
                ts.lastVoxID = thisID;
                ts.lastVoxRefract = mat.refractIndex;
            }
        } else if (ts.lastVoxID != 255u) {
            if (c.refraction) {
                refracted = true;
                rayPos = add(rayPos, muls(rayDir, lastMin + EPS));
                f3 old = rayDir;
                f3 nn = mk(-vox.normal.x, -vox.normal.y, -vox.normal.z);
                settle_normal(hitNormal, nmask, step);
                f3 n = (dot(nn, rayDir) < 0.0f) ? normalize(nn) : hitNormal;
                rayDir = refract(rayDir, n, ts.lastVoxRefract);
                if (rayDir.x == 0.0f && rayDir.y == 0.0f && rayDir.z == 0.0f) rayDir = old;
                inv = mk(1.0f / rayDir.x, 1.0f / rayDir.y, 1.0f / rayDir.z);
                if (!finite_dir(inv)) { count_degenerate(m); c.capped = true; return false; }
                init_dda(rayDir, inv, rayPos, pos, delta, step, side);
                lastMin = 0.0f;
            }
            ts.lastVoxID = 255u;
            ts.lastVoxRefract = 1.0f;
        }
        lastMin = iter_dda_min(delta, step, side, pos, nmask);
        ignoreFirst = false;
    }
    settle_normal(hitNormal, nmask, step);
    return false;
}

// step_map, voxelShared.comp:421-475
static __device__ __forceinline__ bool step_map(RayCtx& c, TState& ts, f3& rayDir, f3 inv, f3& rayPos, bool ignoreFirst,
                                      float maxDepth, f3& hitNormal, Voxel& vox, f3& colorAdd, float& colorMult,
                                      HitInfo& hi)
{
    const DevMap& m = *c.m;
    bool requested = false;
    colorAdd = mk(0.0f, 0.0f, 0.0f);
    colorMult = 1.0f;
    c.c.rays++;
    c.segSteps = 0;
    c.capped = false;
    if (!finite_dir(inv)) { count_degenerate(m); return false; }
    const uint32_t cap = step_cap(m.sx, m.sy, m.sz);
    i3 pos, step; f3 delta, side;
    float lastMin = 0.0f;   // min3(lastSideDist)
    uint32_t nmask = 0;       // stepped axes of the last DDA step whose normal is not yet formed
    init_dda(rayDir, inv, rayPos, pos, delta, step, side);
    while (in_map(m, pos)) {
        if (c.segSteps >= cap) { settle_normal(hitNormal, nmask, step); return false; }
        c.segSteps++;
        c.c.outer++;
        uint32_t t = map_index(m, pos);
        uint32_t w = __ldg(&m.tword[t]);
        uint32_t st = w >> 30;
        if (st == 2u) {
            c.c.entered++;
            if (m.ttouch[t] == 0) m.ttouch[t] = 1;
            float tt = lastMin - EPS;
            f3 up = add(rayPos, muls(rayDir, tt));
            f3 cp = mk((up.x - (float)pos.x) * 8.0f, (up.y - (float)pos.y) * 8.0f, (up.z - (float)pos.z) * 8.0f);
            const float lo = EPS, hi_ = 8.0f - EPS;
            cp.x = gmin(gmax(cp.x, lo), hi_); cp.y = gmin(gmax(cp.y, lo), hi_); cp.z = gmin(gmax(cp.z, lo), hi_);
            bool refracted;
            settle_normal(hitNormal, nmask, step);
            if (step_chunk(c, ts, pos, w & SLOT_MASK, t, rayDir, inv, cp, ignoreFirst, maxDepth, hitNormal, vox,
                           colorAdd, colorMult, refracted, hi)) {
                rayPos = add(mk((float)pos.x, (float)pos.y, (float)pos.z), muls(cp, INV_CHUNK));
                return true;
            }
            if (c.capped) return false;
            if (refracted) {
                rayPos = add(mk((float)pos.x, (float)pos.y, (float)pos.z), muls(cp, INV_CHUNK));
                init_dda(rayDir, inv, rayPos, pos, delta, step, side);
                lastMin = 0.0f;
            }
        } else if (!requested && st != 0u) {
            if (m.treq[t] == 0) m.treq[t] = 1;
            requested = true;
        }
        lastMin = iter_dda_min(delta, step, side, pos, nmask);
        ignoreFirst = false;
    }
    settle_normal(hitNormal, nmask, step);
    return false;
}


__device__ __forceinline__ f3 sky_color(f3 bot, f3 top, f3 dir)
{
    // voxelShared.comp:289-295 gradient branch; mix(x, y, a) = x*(1-a) + y*a
    float a = dir.y * 0.5f + 1.0f;
    return mk(bot.x * (1.0f - a) + top.x * a, bot.y * (1.0f - a) + top.y * a, bot.z * (1.0f - a) + top.z * a);
}

// n-th set bit of a chunk mask -> local position; false if n >= popcount
__device__ __forceinline__ bool select_voxel(const ChunkRec* r, uint32_t n, i3& out, uint32_t& li)
{
    uint32_t count = 0;
    for (uint32_t w = 0; w < 16; w++) {
        uint32_t bits = __ldg(&r->mask[w]);
        uint32_t c = __popc(bits);
        if (count + c > n) {
            for (uint32_t k = n - count; k > 0; k--) bits &= bits - 1u;   // drop the k lowest set bits
            uint32_t b = (uint32_t)(__ffs(bits) - 1);
            uint32_t pos = w * 32u + b;
            li = pos;
            out.x = (int32_t)(pos & 7u); out.y = (int32_t)((pos >> 3) & 7u); out.z = (int32_t)(pos >> 6);
            return true;
        }
        count += c;
    }
    return false;
}

} // namespace dn
