/*
 * dn_light_stream.cuh -- the lighting update as persistent per-lane ray streams.
 *
 * Every lane of a warp owns one voxel at a time and walks that voxel's ray
 * jobs in the reference's order (voxelLighting.comp:238-264):
 *   K specular rays (each up to specBounceLimit segments), then the direct
 *   light rays (K fixed shadow rays, or one along the sun on the first
 *   sample), then numDiffuse diffuse paths (each up to diffuseBounceLimit
 *   segments), then the running average and the write-out.
 * All lanes share one loop whose body is one traversal step of each lane's
 * current ray segment (seg_step: the two-level DDA flattened into one loop), so lanes
 * on different rays, different jobs or different voxels still execute
 * together.  When a segment ends, the lane waits; the per-segment work
 * (shading the finished segment, choosing and setting up the next one,
 * finishing a voxel, fetching the next voxel) runs for all waiting lanes at
 * once when at least `batch` lanes wait (or no lane is still stepping).
 * Each lane accumulates its voxel's sums in exactly the order of the
 * reference loops, so results are bit-identical to the one-voxel-at-a-time
 * form; only the schedule differs.  Voxels are fetched one per lane from a
 * warp-local window over the request list, refilled with one atomic per
 * 32 voxels.
 */
#pragma once
#include "dn_device.cuh"

namespace dn {

#ifndef DN_STREAM_MIN_BLOCKS
#define DN_STREAM_MIN_BLOCKS 4   // 4 blocks of 4 warps per SM (measured best: leaves L1 room for the tile map)
#endif
#ifndef DN_DIFF_MIN_BLOCKS
#define DN_DIFF_MIN_BLOCKS 6     // the diffuse-path kernel (k_light_diffuse): 6 blocks of 4 warps per SM
#endif

enum : uint32_t { PH_FETCH = 0, PH_SPEC = 1, PH_SHADOW = 2, PH_DIFF = 3, PH_FINAL = 4, PH_DONE = 5 };

struct StreamArgs {
    DevMap m;
    const uint32_t* reqs;
    uint32_t* workCounter;
    const uint32_t* nreqPtr;
    const uint32_t* nsamples;
    float4* out;
    unsigned long long* stats;
    uint32_t batch;
    dn_light_params p;
    Material mats[256];
    const struct LightTables* gtab;   // device copy of mats and the shadow directions (k_light_packet)
};

struct MaterialTable { Material m[256]; };

// per-launch tables k_light_packet reads through L1: the materials and the shadow directions
struct LightTables {
    Material mats[256];
    float sdir[65][3];   // shadow directions k < K, [64]: the first-sample direction sunDir + EPS
    float sinv[65][3];
};

// traversal state of one ray segment (flattened two-level DDA, refraction off).  Both levels step with
// the same delta and step signs, so one set of DDA registers (cpos, cside, clastMin) holds the level being
// walked; entering a chunk saves the chunk-level registers (opos, oside, olastMin) and leaving restores
// them.  The reference keeps the side distances before the last step as a vector (lastSideDist) but only
// ever uses its minimum (voxelShared.comp:338, 445), so that minimum is kept instead, formed in the same
// order (min3).
struct Seg {
    f3 pos, dir, inv;
    i3 cpos, opos, step;
    f3 cside, oside, cp;
    float clastMin, olastMin;
    const ChunkRec* rec;
    uint32_t flags;      // bit0 inner level, bit1 ignore (current level), bit2 saved outer ignore, bit3 requested,
                         // bit4 degenerate direction (D16), bit5 the current chunk's materials are all opaque,
                         // bit6 the segment ended on a voxel of such a chunk (hitIdx holds its local index),
                         // bit7 the segment ended on a voxel and pos is not yet its hit position,
                         // bits 8-31 cells visited by the segment (D16 cell cap)
    f3 cadd;
    float cmul;
    TState ts;
};

__device__ __forceinline__ void seg_begin(Seg& s, f3 pos, f3 dir, f3 inv)
{
    // step_map's set-up (voxelShared.comp:421-433) with first voxel ignored
    s.pos = pos; s.dir = dir; s.inv = inv;
    s.cadd = mk(0.0f, 0.0f, 0.0f);
    s.cmul = 1.0f;
    s.ts.lastVoxID = 255u; s.ts.lastVoxRefract = 1.0f;   // D13: fresh per ray job (spec / diffuse bounces keep it)
    f3 delta;
    init_dda(dir, inv, pos, s.cpos, delta, s.step, s.cside);
    s.clastMin = 0.0f;   // min3 of the zero vector
    s.flags = 2u;        // ignore the first voxel
    // D16: a zero or NaN direction component traverses nothing; the first step ends the segment as a miss
    // (a position outside the map) and counts it
    if (!finite_dir(inv)) { s.cpos.x = -1; s.flags = 2u | 16u; }
}

// Enters the loaded chunk of chunk cell idx (tile state cst >= 2) from the chunk level
// (voxelShared.comp:441-449): saves the chunk-level DDA state and starts the voxel-level DDA at the entry point.
__device__ __forceinline__ void seg_enter(Seg& s, const DevMap& m, Counters& c, uint32_t idx, uint32_t cst, f3 delta,
                                          i3 step)
{
    c.outer++;
    c.entered++;
    if (m.ttouch[idx] == 0) m.ttouch[idx] = 1;
    const float tt = s.clastMin - EPS;
    const f3 up = add(s.pos, muls(s.dir, tt));
    f3 cp = mk((up.x - (float)s.cpos.x) * 8.0f, (up.y - (float)s.cpos.y) * 8.0f, (up.z - (float)s.cpos.z) * 8.0f);
    const float lo = EPS, hi_ = 8.0f - EPS;
    // cp is finite here (a finite origin and direction, D16), so fminf / fmaxf give GLSL clamp's values and
    // the floors below are 0..7: a plain conversion, and fl itself for (float)cpos
    cp.x = fminf(fmaxf(cp.x, lo), hi_); cp.y = fminf(fmaxf(cp.y, lo), hi_); cp.z = fminf(fmaxf(cp.z, lo), hi_);
    s.cp = cp;
    s.opos = s.cpos; s.oside = s.cside; s.olastMin = s.clastMin;
    const f3 fl = vfloor(cp);
    s.cpos.x = (int32_t)fl.x; s.cpos.y = (int32_t)fl.y; s.cpos.z = (int32_t)fl.z;
    const f3 sg = mk((float)step.x, (float)step.y, (float)step.z);
    s.cside.x = (sg.x * (fl.x - cp.x) + sg.x * 0.5f + 0.5f) * delta.x;
    s.cside.y = (sg.y * (fl.y - cp.y) + sg.y * 0.5f + 0.5f) * delta.y;
    s.cside.z = (sg.z * (fl.z - cp.z) + sg.z * 0.5f + 0.5f) * delta.z;
    s.clastMin = 0.0f;
    s.rec = &m.rec[__ldg(&m.tword[idx]) & SLOT_MASK];
    // inner level; the chunk inherits ignoreFirst; bit5: the chunk is marked opaque
    s.flags = (s.flags & ~(4u | 32u)) | 1u | ((s.flags & 2u) << 1) | (cst == 3u ? 32u : 0u);
}

// Advances one traversal step.  Returns 0 while the segment continues, 1 on an opaque hit (hit_position()
// moves s.pos to the hit; hitIdx = pool index of the voxel, or its local index in s.rec when flags bit 6 is
// set -- hit_index() gives the pool index), 2 when it leaves the map.  The common case (a chunk cell that is not loaded, or a
// voxel cell that is empty) runs one code path for both levels; entering a chunk, leaving it, reaching a voxel
// and leaving the map are the divergent events.  In a chunk marked 3 in the tile map (every material of its
// voxels opaque under the launch's materials, mark_opaque_word) the first occupied voxel ends the ray without
// its word, rank or material being read: the reference would find it opaque (voxelShared.comp:360-364).
__device__ __forceinline__ uint32_t seg_step(Seg& s, const DevMap& m, const Material* mats, const float* sunStrength,
                                             Counters& c, uint32_t& hitIdx)
{
    const f3 delta = vabs(s.inv);
    const i3 step = s.step;
    const bool inner = (s.flags & 1u) != 0u;
    const uint32_t bx = inner ? 8u : m.sx, by = inner ? 8u : m.sy, bz = inner ? 8u : m.sz;
    const bool inb = (uint32_t)s.cpos.x < bx && (uint32_t)s.cpos.y < by && (uint32_t)s.cpos.z < bz;
    // D16: every visited cell (each outer or inner iteration of step_map / step_chunk) counts; a segment
    // that reached the cap ends as a miss
    if (inb) {
        if (s.flags >= (m.stepCap << 8)) return 2u;   // (flags >> 8) >= stepCap: the low byte holds state bits
        s.flags += 256u;
    }
    const uint32_t idx = (uint32_t)s.cpos.x + bx * ((uint32_t)s.cpos.y + by * (uint32_t)s.cpos.z);
    uint32_t w = 0;
    if (inb) w = __ldg(inner ? &s.rec->mask[idx >> 5] : &m.tbits[idx >> 4]);
    // chunk level: 2-bit state (0 absent, 1 unloaded, 2 loaded); voxel level: occupancy bit -- one shift
    // brings either to the low bits (cst is only read at the chunk level)
    const uint32_t bits = w >> (inner ? (idx & 31u) : ((idx & 15u) << 1));
    const uint32_t cst = bits & 3u;
    const bool occ = inb && (inner ? (((bits & 1u) != 0u) && !(s.flags & 2u)) : (cst >= 2u));
    if (!inb || occ) {
        if (!inner) {
            if (!inb) {
                if (s.flags & 16u) count_degenerate(m);
                return 2u;
            }
            seg_enter(s, m, c, idx, cst, delta, step);
            return 0u;
        }
        if (!inb) {
            // the chunk was crossed without a hit: back to the chunk level, which then iterates
            s.cpos = s.opos; s.cside = s.oside; s.clastMin = s.olastMin;
            s.flags = (s.flags & ~3u) | ((s.flags >> 1) & 2u);
        } else {
            c.inner++;
            c.hits++;
            if (s.flags & 32u) {
                hitIdx = idx;
                s.flags |= 64u | 128u;   // the hit position is formed when shading needs it (hit_position)
                return 1u;
            }
            const uint32_t vi = __ldg(&s.rec->voxBase) + vox_rank(s.rec, idx);
            const uint2 vw = __ldg(&m.vox[vi]);
            const uint32_t material = vw.x >> 24;
            const Material& mat = mats[material];
            if (mat.opacity == 1.0f) {
                hitIdx = vi;
                s.flags |= 128u;
                return 1u;
            }
            const uint32_t thisID = (vw.y & 0xFFFFFF00u) | material;
            if (s.ts.lastVoxID != thisID) {
                const f3 alb = mk((float)((vw.y >> 24) & 0xFF) * INV255, (float)((vw.y >> 16) & 0xFF) * INV255,
                                  (float)((vw.y >> 8) & 0xFF) * INV255);
                const float k = s.cmul * mat.opacity;
                s.cadd.x = s.cadd.x + k * alb.x * sunStrength[0];
                s.cadd.y = s.cadd.y + k * alb.y * sunStrength[1];
                s.cadd.z = s.cadd.z + k * alb.z * sunStrength[2];
                s.cmul = s.cmul * (1.0f - mat.opacity);
                s.ts.lastVoxID = thisID;
                s.ts.lastVoxRefract = mat.refractIndex;
            }
        }
    } else {
        // an empty cell, either level, without branches: the counters, and at the voxel level the end of a
        // run of transparent voxels (lastVoxID 255 always comes with refract 1, so writing both is the
        // reference's reset); an unloaded chunk cell requests its chunk once per ray
        c.inner += inner ? 1u : 0u;
        c.outer += inner ? 0u : 1u;
        s.ts.lastVoxID = inner ? 255u : s.ts.lastVoxID;
        s.ts.lastVoxRefract = inner ? 1.0f : s.ts.lastVoxRefract;
        if (!inner && !(s.flags & 8u) && cst != 0u) {
            if (m.treq[idx] == 0) m.treq[idx] = 1;
            s.flags |= 8u;
        }
    }
    // iterate_DDA on the current level (voxelShared.comp:309-317).  With a finite direction (D16) every side
    // distance is finite and non-negative (never -0), so fminf gives GLSL min's value (y < x ? y : x) and
    // adding delta only on the stepped axes gives exactly side + (mask ? 1 : 0) * delta.
    const float gyz = fminf(s.cside.y, s.cside.z), gzx = fminf(s.cside.z, s.cside.x), gxy = fminf(s.cside.x, s.cside.y);
    s.clastMin = fminf(gxy, s.cside.z);   // min3(lastSideDist) of the next step
    const bool mx = s.cside.x <= gyz;
    const bool my = s.cside.y <= gzx;
    const bool mz = s.cside.z <= gxy;
    if (mx) s.cside.x = s.cside.x + delta.x;
    if (my) s.cside.y = s.cside.y + delta.y;
    if (mz) s.cside.z = s.cside.z + delta.z;
    s.cpos.x += (int32_t)mx * step.x; s.cpos.y += (int32_t)my * step.y; s.cpos.z += (int32_t)mz * step.z;
    s.flags &= ~2u;
    return 0u;
}

__device__ __forceinline__ f3 rcp3(f3 d) { return mk(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)); }

// the pool index of the voxel a segment ended on (seg_step's hitIdx)
__device__ __forceinline__ uint32_t hit_index(const Seg& s, uint32_t hitIdx)
{
    return (s.flags & 64u) ? __ldg(&s.rec->voxBase) + vox_rank(s.rec, hitIdx) : hitIdx;
}

// the hit position of a segment that ended on a voxel (voxelShared.comp:362-364), formed when shading needs
// it: shadow rays never do.  The segment's state is unchanged since the hit.
__device__ __forceinline__ void hit_position(Seg& s)
{
    if (s.flags & 128u) {
        const float t = s.clastMin + EPS;
        const f3 cp = add(s.cp, muls(s.dir, t));
        s.pos = add(mk((float)s.opos.x, (float)s.opos.y, (float)s.opos.z), muls(cp, INV_CHUNK));
        s.flags &= ~128u;
    }
}

// per-lane job state of the voxel being lit
struct Job {
    uint32_t phase, k, b, i;
    uint32_t req, vlane, vidx;      // request, lane within it, pool index of the voxel
    f3 pos0, tnormal, talbedo, refl;
    uint32_t tmat, key;
    float indirect;
    bool firstSample, doSpec, doDiff;
    f3 spec, direct, acc;           // acc: shadow sum, then diffuse sum
    f3 jA, jB, jC;                  // spec: mult, lastPos ; diffuse: nc, hitNormal, lastDir
    uint32_t jU;                    // spec: reflectType ; diffuse: material of the last hit
    uint32_t map;                   // many-map launches: the voxel's map
};

} // namespace dn

namespace dn {

__device__ __forceinline__ uint32_t lane_id_s()
{
    uint32_t l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

struct StreamShared {
    Material mats[256];
    float sdir[65][3];   // shadow directions k < K, [64]: the first-sample direction sunDir + EPS
    float sinv[65][3];
};


// diffuse bounce direction (voxelLighting.comp:160-168)
__device__ __forceinline__ f3 diffuse_dir(const Job& j, const dn_light_params& p, const Material* mats, bool rngSin)
{
    const Material& hm = mats[j.jU];
    bool lobe = false;
    const float seed = p.time * (float)(j.i + 1u);
    if (j.b > 0) {
        const float r = rngSin ? srand1(seed + (float)p.diffuseBounceLimit + (float)j.b)
                               : hrand(j.key, 2u, (j.i * 16u + j.b) << 8);
        lobe = (r + 1.0f) * 0.5f < hm.specular;
    }
    if (lobe) {
        const f3 rs = rngSin ? sphere_sin(p.time + (float)j.b) : sphere_hash(j.key, 3u, j.i * 16u + j.b);
        return normalize(add(muls(reflect(j.jC, j.jB), (float)hm.shininess), rs));
    }
    if (j.firstSample) return adds(normalize(j.jB), EPS);
    const f3 rs = rngSin ? sphere_sin(seed + (float)j.b) : sphere_hash(j.key, 1u, j.i * 16u + j.b);
    return adds(normalize(add(j.jB, rs)), EPS);
}

// Consumes the finished segment (hitState 1 hit / 2 miss) and sets up the next segment of this lane's
// voxel; returns true when a segment was started.  Leaves the job in PH_FETCH when the voxel is done.
// DIFFONLY: the voxel's diffuse paths only (its specular and direct light came from the ray-fan kernel,
// which left the direct light in the diffuse output slot); the final write replaces that slot with the
// voxel's new diffuse lighting and leaves the specular slot and the lit-voxel count alone.
template <bool DIFFONLY = false>
__device__ __forceinline__ bool advance(Job& j, Seg& s, uint32_t& hitState, uint32_t hitIdx, const DevMap& m,
                                        const dn_light_params& p, const Material* mats, const float (*sdir)[3],
                                        const float (*sinv)[3], float4* out, Counters& c, uint32_t& lit)
{
    const bool rngSin = p.rngMode == 1u;
    const f3 sun = mk(p.sunStrength[0], p.sunStrength[1], p.sunStrength[2]);
    const f3 sunDir = mk(p.sunDir[0], p.sunDir[1], p.sunDir[2]);
    if (hitState) {
        const bool hit = hitState == 1u;
        hitState = 0;
        Voxel hv;
        if (hit) hit_position(s);
        if (hit) decompress(m, hit_index(s, hitIdx), hv);
        // the diffuse-only kernel's jobs never reach the specular and shadow phases: with DIFFONLY their
        // code is left out of it (a smaller kernel: fewer instruction-fetch stalls)
        if (!DIFFONLY && j.phase == PH_SPEC) {
            // specular_ray body after step_map (voxelLighting.comp:98-144)
            bool done = true;
            if (hit) {
                const i3 hp{f2i(truncf(s.pos.x)), f2i(truncf(s.pos.y)), f2i(truncf(s.pos.z))};
                if (in_map(m, hp)) {
                    uint8_t* vp = &m.tvis[map_index(m, hp)];
                    if (*vp == 0) *vp = 1;
                }
                const f3 d = vabs(sub(vfloor(muls(s.pos, 8.0f)), vfloor(muls(j.jB, 8.0f))));
                if (!(dot(d, d) <= 1.0f)) {
                    const Material& hm = mats[hv.material];
                    const f3 hd = muls(hv.diff, 1.0f - hm.specular);
                    if (hm.emissive) {
                        j.spec.x = j.spec.x + ((hv.albedo.x * p.emissiveStrength * s.cmul + s.cadd.x) * j.jA.x) * j.talbedo.x;
                        j.spec.y = j.spec.y + ((hv.albedo.y * p.emissiveStrength * s.cmul + s.cadd.y) * j.jA.y) * j.talbedo.y;
                        j.spec.z = j.spec.z + ((hv.albedo.z * p.emissiveStrength * s.cmul + s.cadd.z) * j.jA.z) * j.talbedo.z;
                    } else {
                        const f3 hc = mul(hd, hv.albedo);
                        j.spec.x = j.spec.x + (hc.x * s.cmul + s.cadd.x) * j.jA.x;
                        j.spec.y = j.spec.y + (hc.y * s.cmul + s.cadd.y) * j.jA.y;
                        j.spec.z = j.spec.z + (hc.z * s.cmul + s.cadd.z) * j.jA.z;
                        if (hm.specular != 0.0f) {
                            j.jA.x = j.jA.x * (hv.albedo.x * s.cmul * hm.specular);
                            j.jA.y = j.jA.y * (hv.albedo.y * s.cmul * hm.specular);
                            j.jA.z = j.jA.z * (hv.albedo.z * s.cmul * hm.specular);
                            j.jU = hm.reflectType;
                            j.jB = s.pos;
                            const f3 nd = reflect(s.dir, hv.normal);
                            j.b++;
                            if (j.b < p.specBounceLimit) {
                                const TState keep = s.ts;
                                seg_begin(s, s.pos, nd, rcp3(nd));   // next bounce
                                s.ts = keep;      // one ray job: bounces keep the transparency state
                                c.rays++;
                                return true;
                            }
                        }
                    }
                }
            } else if (dot(s.dir, sunDir) > 0.99f) {
                j.spec.x = j.spec.x + (sun.x * s.cmul + s.cadd.x);
                j.spec.y = j.spec.y + (sun.y * s.cmul + s.cadd.y);
                j.spec.z = j.spec.z + (sun.z * s.cmul + s.cadd.z);
            } else {
                const f3 sc = (j.jU == 1u) ? sky_color(mk(p.skyBot[0], p.skyBot[1], p.skyBot[2]),
                                                      mk(p.skyTop[0], p.skyTop[1], p.skyTop[2]), s.dir) : sun;
                j.spec.x = j.spec.x + (sc.x * s.cmul + s.cadd.x) * j.jA.x;
                j.spec.y = j.spec.y + (sc.y * s.cmul + s.cadd.y) * j.jA.y;
                j.spec.z = j.spec.z + (sc.z * s.cmul + s.cadd.z) * j.jA.z;
            }
            if (done) { j.k++; j.b = 0; }
        } else if (!DIFFONLY && j.phase == PH_SHADOW) {
            if (!hit) {
                j.acc.x = j.acc.x + (sun.x * s.cmul + s.cadd.x);
                j.acc.y = j.acc.y + (sun.y * s.cmul + s.cadd.y);
                j.acc.z = j.acc.z + (sun.z * s.cmul + s.cadd.z);
            }
            j.k++;
        } else if (j.phase == PH_DIFF) {
            // diffuse_ray body after step_map (voxelLighting.comp:176-201)
            bool pathDone = true;
            if (hit) {
                j.jB = hv.normal;
                j.jU = hv.material;
                const f3 d = vabs(sub(vfloor(muls(j.pos0, 8.0f)), vfloor(muls(s.pos, 8.0f))));
                if (!(dot(d, d) < 1.0f)) {
                    const Material& hm = mats[hv.material];
                    if (hm.emissive) {
                        j.acc.x = j.acc.x + j.jA.x * (hv.albedo.x * p.emissiveStrength * s.cmul + s.cadd.x);
                        j.acc.y = j.acc.y + j.jA.y * (hv.albedo.y * p.emissiveStrength * s.cmul + s.cadd.y);
                        j.acc.z = j.acc.z + j.jA.z * (hv.albedo.z * p.emissiveStrength * s.cmul + s.cadd.z);
                    } else {
                        j.jA.x = j.jA.x * (hv.albedo.x * s.cmul + s.cadd.x);
                        j.jA.y = j.jA.y * (hv.albedo.y * s.cmul + s.cadd.y);
                        j.jA.z = j.jA.z * (hv.albedo.z * s.cmul + s.cadd.z);
                        j.jC = s.dir;
                        j.b++;
                        if (j.b < p.diffuseBounceLimit) {
                            const f3 nd = diffuse_dir(j, p, mats, rngSin);
                            const TState keep = s.ts;
                            seg_begin(s, s.pos, nd, rcp3(nd));
                            s.ts = keep;
                            c.rays++;
                            return true;
                        }
                    }
                }
            } else {
                const float k = gmax(dot(s.dir, sunDir), 0.0f);
                j.acc.x = j.acc.x + (j.jA.x * k * sun.x * s.cmul + s.cadd.x);
                j.acc.y = j.acc.y + (j.jA.y * k * sun.y * s.cmul + s.cadd.y);
                j.acc.z = j.acc.z + (j.jA.z * k * sun.z * s.cmul + s.cadd.z);
            }
            if (pathDone) { j.acc = add(j.acc, j.direct); j.i++; j.b = 0; }
        }
    }
    // start the next segment of this voxel
    for (int guard = 0; guard < 8; guard++) {
        if (!DIFFONLY && j.phase == PH_SPEC) {
            if (j.k < p.K) {
                if (p.specBounceLimit == 0u) { j.k++; continue; }
                const Material& tm = mats[j.tmat];
                j.b = 0; j.jA = j.talbedo; j.jB = j.pos0; j.jU = tm.reflectType;
                const f3 P = mk(p.spherePts[j.k][0], p.spherePts[j.k][1], p.spherePts[j.k][2]);
                const f3 sd = adds(normalize(add(muls(j.refl, (float)tm.shininess), P)), EPS);
                seg_begin(s, j.pos0, sd, rcp3(sd));
                c.rays++;
                return true;
            }
            j.spec = divs(j.spec, (float)p.K);
            j.phase = j.doDiff ? PH_SHADOW : PH_FINAL;
            j.k = 0;
            continue;
        }
        if (!DIFFONLY && j.phase == PH_SHADOW) {
            const uint32_t n = j.firstSample ? 1u : p.K;
            if (j.k < n) {
                const uint32_t q = j.firstSample ? 64u : j.k;
                seg_begin(s, j.pos0, mk(sdir[q][0], sdir[q][1], sdir[q][2]), mk(sinv[q][0], sinv[q][1], sinv[q][2]));
                c.rays++;
                return true;
            }
            j.direct = divs(j.acc, (float)n);
            j.acc = mk(0.0f, 0.0f, 0.0f);
            j.phase = PH_DIFF;
            j.i = 0; j.b = 0;
            continue;
        }
        if (j.phase == PH_DIFF) {
            if (j.i < p.numDiffuse) {
                if (j.b == 0) {
                    const f3 amb = mk(p.ambient[0], p.ambient[1], p.ambient[2]);
                    j.acc = add(j.acc, amb);
                    if (p.diffuseBounceLimit == 0u) { j.acc = add(j.acc, j.direct); j.i++; continue; }
                    j.jA = mk(1.0f, 1.0f, 1.0f);
                    j.jB = adds(j.tnormal, EPS);
                    j.jC = mk(0.0f, 0.0f, 0.0f);
                    j.jU = j.tmat;
                }
                const f3 nd = diffuse_dir(j, p, mats, rngSin);
                seg_begin(s, j.pos0, nd, rcp3(nd));
                c.rays++;
                return true;
            }
            const float4 prev = __ldg(&m.diff[j.vidx]);
            const float den = j.indirect + (float)p.numDiffuse;
            j.acc.x = (prev.x * j.indirect + j.acc.x) / den;
            j.acc.y = (prev.y * j.indirect + j.acc.y) / den;
            j.acc.z = (prev.z * j.indirect + j.acc.z) / den;
            j.phase = PH_FINAL;
            continue;
        }
        if (j.phase == PH_FINAL) {
            const float4 outS = make_float4(gmin(gmax(j.spec.x, 0.0f), 1.0f), gmin(gmax(j.spec.y, 0.0f), 1.0f),
                                            gmin(gmax(j.spec.z, 0.0f), 1.0f), 0.0f);
            const float4 outD = make_float4(gmin(gmax(j.acc.x, 0.0f), 1.0f), gmin(gmax(j.acc.y, 0.0f), 1.0f),
                                            gmin(gmax(j.acc.z, 0.0f), 1.0f), 0.0f);
            const uint64_t o = ((uint64_t)j.req * 32u + j.vlane) * 2u;
            out[o] = outD;
            if constexpr (!DIFFONLY) {
                out[o + 1] = outS;
                lit++;
            }
            j.phase = PH_FETCH;
        }
        return false;
    }
    return false;
}

// Sets up voxel (req, vlane); returns false (and writes zero outputs) when the slot holds no voxel.
// DIFFONLY: false (writing nothing) also for a voxel without diffuse paths; otherwise the job starts at its
// diffuse paths with the direct light the ray-fan kernel left in the voxel's diffuse output slot.
template <bool DIFFONLY = false>
__device__ __forceinline__ bool voxel_setup(Job& j, uint32_t req, uint32_t vlane, const DevMap& m, const dn_light_params& p,
                                            const Material* mats, const uint32_t* reqs, const uint32_t* nsamples, float4* out)
{
    j.req = req; j.vlane = vlane;
    const uint32_t word = reqs[req];
    const uint32_t tile = word >> 4, group = word & 15u;
    const uint32_t tw = __ldg(&m.tword[tile]);
    const uint32_t vn = group * 32u + vlane;
    i3 cp; uint32_t li;
    const ChunkRec* rc = &m.rec[tw & SLOT_MASK];
    if ((tw >> 30) != 2u || vn >= __ldg(&rc->nvox) || !select_voxel(rc, vn, cp, li)) {
        if constexpr (!DIFFONLY) {
            const uint64_t o = ((uint64_t)req * 32u + vlane) * 2u;
            out[o] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            out[o + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        return false;
    }
    const i3 mp{__ldg(&rc->pos[0]), __ldg(&rc->pos[1]), __ldg(&rc->pos[2])};
    j.vidx = __ldg(&rc->voxBase) + vn;
    const uint2 w = __ldg(&m.vox[j.vidx]);
    j.tnormal = mk(((float)((w.x >> 16) & 0xFF) * INV255 - 0.5f) * 2.0f, ((float)((w.x >> 8) & 0xFF) * INV255 - 0.5f) * 2.0f,
                   ((float)(w.x & 0xFF) * INV255 - 0.5f) * 2.0f);
    j.tmat = w.x >> 24;
    j.talbedo = mk((float)((w.y >> 24) & 0xFF) * INV255, (float)((w.y >> 16) & 0xFF) * INV255,
                   (float)((w.y >> 8) & 0xFF) * INV255);
    const uint32_t samples = __ldg(&nsamples[tw & SLOT_MASK]);
    const uint32_t ns = samples < p.maxDiffuse ? samples : p.maxDiffuse;
    j.indirect = (float)ns;
    j.firstSample = (j.indirect == 0.0f);
    const uint32_t gx = (uint32_t)(mp.x * 8 + cp.x), gy = (uint32_t)(mp.y * 8 + cp.y), gz = (uint32_t)(mp.z * 8 + cp.z);
    j.key = rng_key(__float_as_uint(p.time), p.mapId, gx + (m.sx * 8u) * (gy + (m.sy * 8u) * gz));
    f3 rp;
    rp.x = INV_CHUNK * (float)cp.x + (float)mp.x + HALF_INV_CHUNK;
    rp.y = INV_CHUNK * (float)cp.y + (float)mp.y + HALF_INV_CHUNK;
    rp.z = INV_CHUNK * (float)cp.z + (float)mp.z + HALF_INV_CHUNK;
    const float off = HALF_INV_CHUNK - EPS;
    j.pos0 = add(rp, muls(j.tnormal, off));
    const Material& tm = mats[j.tmat];
    j.doDiff = tm.specular < 1.0f;
    if constexpr (DIFFONLY) {
        if (!j.doDiff) return false;
        const float4 d = out[((uint64_t)req * 32u + vlane) * 2u];
        j.direct = mk(d.x, d.y, d.z);
        j.spec = mk(0.0f, 0.0f, 0.0f); j.acc = j.spec;
        j.k = 0; j.b = 0; j.i = 0;
        j.phase = PH_DIFF;
        return true;
    }
    const f3 viewDir = sub(j.pos0, mk(p.camPos[0], p.camPos[1], p.camPos[2]));
    j.doSpec = tm.specular > 0.0f && dot(viewDir, j.tnormal) < 0.0f && tm.reflectType <= 1u;
    if (j.doSpec) j.refl = reflect(normalize(viewDir), j.tnormal);
    j.spec = mk(0.0f, 0.0f, 0.0f); j.acc = j.spec; j.direct = j.spec;
    j.k = 0; j.b = 0; j.i = 0;
    j.phase = j.doSpec ? PH_SPEC : (j.doDiff ? PH_SHADOW : PH_FINAL);
    return true;
}

// ------------------------------------------------------------ launches

// one map of a many-map lighting launch (device memory, written by the host and by k_batch_prep)
struct BatchLightMap {
    DevMap m;
    const uint32_t* reqs;
    const uint32_t* nsamples;
    float4* out;
    uint32_t* nreqPtr;          // the map's request count (clamped by k_batch_prep)
    uint64_t reqCap;
    dn_light_params p;
    const Material* mats;       // the map's 256 materials
    float4* diffOut;            // committed lighting and sample counts (k_commit_batch)
    float4* specOut;
    uint32_t* samplesOut;
    float sdir[65][3];          // shadow directions of this map (k_batch_prep)
    float sinv[65][3];
};

struct BatchLightArgs {
    BatchLightMap* maps;
    const uint32_t* reqStart;   // [nmaps + 1]: first request of each map in the launch's queue
    uint32_t nmaps;
    uint32_t* workCounter;
    unsigned long long* stats;
    uint32_t batch;
};

// shadow directions normalize(sunDir * softness + P_k) + EPS (k < K) and sunDir + EPS ([64]) with reciprocals
__device__ __forceinline__ void shadow_dir(const dn_light_params& p, int k, float* d3, float* i3)
{
    const f3 sd = mk(p.sunDir[0], p.sunDir[1], p.sunDir[2]);
    f3 d;
    if (k == 64) d = adds(sd, EPS);
    else if ((uint32_t)k < p.K) {
        const f3 P = mk(p.spherePts[k][0], p.spherePts[k][1], p.spherePts[k][2]);
        d = adds(normalize(add(muls(sd, p.shadowSoftness), P)), EPS);
    } else d = mk(1.0f, 1.0f, 1.0f);
    d3[0] = d.x; d3[1] = d.y; d3[2] = d.z;
    i3[0] = __frcp_rn(d.x); i3[1] = __frcp_rn(d.y); i3[2] = __frcp_rn(d.z);
}

// The persistent loop of a lighting launch.  MANY = false: one map whose arguments live in the launch's
// parameter space (one) and whose materials and shadow directions were staged into sh.  MANY = true: a
// queue over the requests of many maps (many); each lane reads its current voxel's map, parameters,
// materials and shadow directions from that map's entry of the device table.  DIFFONLY: the
// diffuse paths of the voxels the ray-fan kernel lit (advance<true>); one map's materials are read from
// its device tables (one->gtab) and sh is not used.
template <bool MANY, bool DIFFONLY = false>
__device__ __forceinline__ void stream_loop(const StreamArgs* one, const BatchLightArgs* many, const StreamShared* sh,
                                            Job& j)
{
    const uint32_t lane = lane_id_s();
    const uint32_t batch = MANY ? many->batch : one->batch;
    uint32_t nreq = 0;
    if constexpr (MANY) nreq = *(volatile const uint32_t*)&many->reqStart[many->nmaps];
    else nreq = *(volatile const uint32_t*)one->nreqPtr;
    uint32_t* const counter = MANY ? many->workCounter : one->workCounter;
    uint32_t winMap = 0, winReq = 0, winNext = 32;     // warp-uniform voxel window: map, request, next lane in it
    bool exhausted = false;
    j.phase = PH_FETCH;
    j.map = 0;
    // the lane's current map (MANY only), read through its table entry: a register copy of the map's
    // arguments spilled 228 bytes per thread, and the pointer measured +1.2 % on the 64-map workload
    const BatchLightMap* le = nullptr;
    uint32_t lmi = 0xFFFFFFFFu;
    if constexpr (MANY) { le = &many->maps[0]; lmi = 0; }
    auto M = [&]() -> const DevMap& { if constexpr (MANY) return le->m; else return one->m; };
    auto P = [&]() -> const dn_light_params& { if constexpr (MANY) return le->p; else return one->p; };
    auto MATS = [&]() -> const Material* {
        if constexpr (MANY) return le->mats;
        else if constexpr (DIFFONLY) return one->gtab->mats;
        else return sh->mats;
    };
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
                        if (!exhausted && lane == 0) r = atomicAdd(counter, 1u);
                        r = __shfl_sync(0xFFFFFFFFu, r, 0);
                        if (exhausted || r >= nreq) {
                            exhausted = true;
                            if (j.phase == PH_FETCH) j.phase = PH_DONE;
                            break;
                        }
                        if constexpr (MANY) {
                            // the map whose request range holds r: reqStart[map] <= r < reqStart[map + 1]
                            uint32_t lo = 0, hi = many->nmaps;
                            while (hi - lo > 1u) {
                                const uint32_t mid = (lo + hi) >> 1;
                                if (__ldg(&many->reqStart[mid]) <= r) lo = mid; else hi = mid;
                            }
                            winMap = lo;
                            winReq = r - __ldg(&many->reqStart[lo]);
                        } else {
                            winReq = r;
                        }
                        winNext = 0;
                    }
                    const uint32_t rank = __popc(need & ((1u << lane) - 1u));
                    if (j.phase == PH_FETCH && winNext + rank < 32u) {
                        if constexpr (MANY) {
                            const BatchLightMap& e = many->maps[winMap];
                            if (winMap != lmi) { le = &e; lmi = winMap; }
                            j.map = winMap;
                            voxel_setup<DIFFONLY>(j, winReq, winNext + rank, e.m, e.p, e.mats, e.reqs, e.nsamples, e.out);
                        } else {
                            voxel_setup<DIFFONLY>(j, winReq, winNext + rank, one->m, one->p, MATS(), one->reqs, one->nsamples,
                                                  one->out);
                        }
                    }
                    const uint32_t took = (uint32_t)__popc(need) < 32u - winNext ? (uint32_t)__popc(need) : 32u - winNext;
                    winNext += took;
                }
                // shade the finished segment and set up the next one (or finish the voxel)
                if (!rayActive && j.phase != PH_DONE && j.phase != PH_FETCH) {
                    if constexpr (MANY) {
                        if (j.map != lmi) { le = &many->maps[j.map]; lmi = j.map; }
                        rayActive = advance<DIFFONLY>(j, s, hitState, hitIdx, le->m, le->p, le->mats, le->sdir, le->sinv, le->out,
                                                      c, lit);
                    } else if constexpr (DIFFONLY) {
                        rayActive = advance<true>(j, s, hitState, hitIdx, one->m, one->p, MATS(), one->gtab->sdir,
                                                  one->gtab->sinv, one->out, c, lit);
                    } else {
                        rayActive = advance(j, s, hitState, hitIdx, one->m, one->p, sh->mats, sh->sdir, sh->sinv, one->out, c, lit);
                    }
                }
                if (__ballot_sync(0xFFFFFFFFu, j.phase == PH_FETCH) == 0u) break;
            }
        }
        if (rayActive) {
            const uint32_t r = seg_step(s, M(), MATS(), P().sunStrength, c, hitIdx);
            if (r) { rayActive = false; hitState = r; }
        }
    }
    flush_counters(MANY ? many->stats : one->stats, c, 0, lit);
}

} // namespace dn
