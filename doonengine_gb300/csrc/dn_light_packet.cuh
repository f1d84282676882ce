/*
 * dn_light_packet.cuh -- the lighting update with ray fans traced as warp packets.
 *
 * Every lit voxel casts two fans of K rays from one point: K specular rays around its reflection
 * direction (voxelLighting.comp:83-146, each up to specBounceLimit segments) and K shadow rays around the
 * sun direction (D8).  A warp takes one request group (32 voxels of one chunk) and traces each voxel's
 * fan across its lanes -- lane k traces ray k, 32/K voxels per pass when K <= 32, ceil(K/32) rounds when
 * K > 32 -- so the lanes of a warp walk nearly the same cells in the same order: the shadow rays of a
 * voxel are almost parallel, and the specular rays share their origin and lobe.  The per-voxel sums are
 * then formed by a serial walk over the lanes in ray order (shuffles / shared memory), so every sum is
 * accumulated in exactly the reference's order.  The diffuse paths (numDiffuse per voxel, up to
 * diffuseBounceLimit segments each) run one lane per voxel, and each lane finishes its voxel as the
 * reference's lighting main does (running average, clamps, voxelLighting.comp:238-288).
 *
 * Results, traversal side effects (requested / touched / visible flags) and counters are those of the
 * one-voxel-per-lane forms (dn_light.cuh, dn_light_stream.cuh): the same rays are traced with the same
 * operations; only the assignment of rays to lanes differs.
 */
#pragma once
#include "dn_light_stream.cuh"

namespace dn {

#ifndef DN_PACKET_MIN_BLOCKS
#define DN_PACKET_MIN_BLOCKS 4
#endif

constexpr uint32_t PK_MAX_SPEC_SEGMENTS = 4;   // specBounceLimit handled here; larger limits use the stream kernel

// per-voxel data of the warp's request group (shared memory, written by the voxel's lane)
struct PacketVoxel {
    f3 pos0, tnormal, talbedo, refl;
    f3 spec;                 // specular sum / K (after the specular pass)
    f3 direct;               // shadow sum / n (after the shadow pass)
    uint32_t tmat, key, vidx, flags;   // flags: 1 valid, 2 first sample, 4 specular pass, 8 diffuse passes
    float indirect;
};
enum : uint32_t { PV_VALID = 1u, PV_FIRST = 2u, PV_SPEC = 4u, PV_DIFF = 8u };

struct PacketWarp {
    PacketVoxel v[32];
    float con[32][PK_MAX_SPEC_SEGMENTS][3];   // specular contributions of each lane's ray, in segment order
    uint32_t ncon[32];
};

// sets up voxel (req, lane) of the group (voxel_setup of dn_light_stream.cuh); invalid slots get zero output
__device__ __forceinline__ void packet_setup(PacketVoxel& pv, uint32_t req, uint32_t lane, const DevMap& m,
                                             const dn_light_params& p, const Material* mats, const uint32_t* reqs,
                                             const uint32_t* nsamples, float4* out)
{
    pv.flags = 0;
    const uint32_t word = reqs[req];
    const uint32_t tile = word >> 4, group = word & 15u;
    const uint32_t tw = __ldg(&m.tword[tile]);
    const uint32_t vn = group * 32u + lane;
    i3 cp; uint32_t li;
    const ChunkRec* rc = &m.rec[tw & SLOT_MASK];
    if ((tw >> 30) != 2u || vn >= __ldg(&rc->nvox) || !select_voxel(rc, vn, cp, li)) {
        const uint64_t o = ((uint64_t)req * 32u + lane) * 2u;
        out[o] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        out[o + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const i3 mp{__ldg(&rc->pos[0]), __ldg(&rc->pos[1]), __ldg(&rc->pos[2])};
    pv.vidx = __ldg(&rc->voxBase) + vn;
    const uint2 w = __ldg(&m.vox[pv.vidx]);
    pv.tnormal = mk(((float)((w.x >> 16) & 0xFF) * INV255 - 0.5f) * 2.0f, ((float)((w.x >> 8) & 0xFF) * INV255 - 0.5f) * 2.0f,
                    ((float)(w.x & 0xFF) * INV255 - 0.5f) * 2.0f);
    pv.tmat = w.x >> 24;
    pv.talbedo = mk((float)((w.y >> 24) & 0xFF) * INV255, (float)((w.y >> 16) & 0xFF) * INV255,
                    (float)((w.y >> 8) & 0xFF) * INV255);
    const uint32_t samples = __ldg(&nsamples[tw & SLOT_MASK]);
    const uint32_t ns = samples < p.maxDiffuse ? samples : p.maxDiffuse;
    pv.indirect = (float)ns;
    const bool first = (pv.indirect == 0.0f);
    const uint32_t gx = (uint32_t)(mp.x * 8 + cp.x), gy = (uint32_t)(mp.y * 8 + cp.y), gz = (uint32_t)(mp.z * 8 + cp.z);
    pv.key = rng_key(__float_as_uint(p.time), p.mapId, gx + (m.sx * 8u) * (gy + (m.sy * 8u) * gz));
    f3 rp;
    rp.x = INV_CHUNK * (float)cp.x + (float)mp.x + HALF_INV_CHUNK;
    rp.y = INV_CHUNK * (float)cp.y + (float)mp.y + HALF_INV_CHUNK;
    rp.z = INV_CHUNK * (float)cp.z + (float)mp.z + HALF_INV_CHUNK;
    const float off = HALF_INV_CHUNK - EPS;
    pv.pos0 = add(rp, muls(pv.tnormal, off));
    const Material& tm = mats[pv.tmat];
    const f3 viewDir = sub(pv.pos0, mk(p.camPos[0], p.camPos[1], p.camPos[2]));
    const bool doSpec = tm.specular > 0.0f && dot(viewDir, pv.tnormal) < 0.0f && tm.reflectType <= 1u;
    const bool doDiff = tm.specular < 1.0f;
    if (doSpec) pv.refl = reflect(normalize(viewDir), pv.tnormal);
    pv.spec = mk(0.0f, 0.0f, 0.0f);
    pv.direct = pv.spec;
    pv.flags = PV_VALID | (first ? PV_FIRST : 0u) | (doSpec ? PV_SPEC : 0u) | (doDiff ? PV_DIFF : 0u);
}

// steps every lane's current segment until all of them ended (hs: 1 hit, 2 miss)
__device__ __forceinline__ void packet_trace(bool stepping, Seg& s, const DevMap& m, const Material* mats,
                                             const float* sun, Counters& c, uint32_t& hs, uint32_t& hitIdx)
{
    while (__any_sync(0xFFFFFFFFu, stepping)) {
        if (stepping) {
            const uint32_t r = seg_step(s, m, mats, sun, c, hitIdx);
            if (r) { stepping = false; hs = r; }
        }
    }
}

// the k-th lane of segment sg of a pass over the voxels of 'mask': voxel index (or -1) and ray index
__device__ __forceinline__ int pass_voxel(uint32_t mask, uint32_t base, uint32_t K, uint32_t lane, uint32_t round,
                                          uint32_t& kk, uint32_t& sg)
{
    const uint32_t vpp = K <= 32u ? 32u / K : 1u;
    sg = K <= 32u ? lane / K : 0u;
    kk = K <= 32u ? lane - sg * K : lane + 32u * round;
    const uint32_t n = (uint32_t)__popc(mask);
    if (sg >= vpp || base + sg >= n || kk >= K) return -1;
    // the (base + sg)-th set bit of mask
    uint32_t mm = mask;
    for (uint32_t t = 0; t < base + sg; t++) mm &= mm - 1u;
    return __ffs(mm) - 1;
}

enum : uint32_t { PP_SPEC = 0, PP_FIRST = 1, PP_FAN = 2, PP_DIFF = 3, PP_DONE = 4 };

// The request groups of one launch.  Per group the warp runs four passes -- specular fans, first-sample
// shadow rays, shadow fans, diffuse paths -- as a state machine around a single stepping loop: each pass
// unit (a pack of voxels for the fans, all voxels for the others) starts one segment per lane, the lanes
// step together until every segment ended, the pass shades the ended segments and starts follow-up
// segments, and when no lane has work the unit's sums are formed and the next unit starts.
template <bool MANY>
__device__ __forceinline__ void packet_loop(const StreamArgs* one, const BatchLightArgs* many, const StreamShared* sh,
                                            PacketWarp& W)
{
    const uint32_t lane = lane_id_s();
    uint32_t nreq = 0;
    if constexpr (MANY) nreq = *(volatile const uint32_t*)&many->reqStart[many->nmaps];
    else nreq = *(volatile const uint32_t*)one->nreqPtr;
    uint32_t* const counter = MANY ? many->workCounter : one->workCounter;
    Counters c{0, 0, 0, 0, 0};
    uint32_t lit = 0;
    for (;;) {
        uint32_t r = 0;
        if (lane == 0) r = atomicAdd(counter, 1u);
        r = __shfl_sync(0xFFFFFFFFu, r, 0);
        if (r >= nreq) break;
        // the group's map (warp-uniform)
        const BatchLightMap* e = nullptr;
        uint32_t req = r;
        if constexpr (MANY) {
            uint32_t lo = 0, hi = many->nmaps;
            while (hi - lo > 1u) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldg(&many->reqStart[mid]) <= r) lo = mid; else hi = mid;
            }
            e = &many->maps[lo];
            req = r - __ldg(&many->reqStart[lo]);
        }
        const DevMap& m = MANY ? e->m : one->m;
        const dn_light_params& p = MANY ? e->p : one->p;
        const Material* mats = MANY ? e->mats : sh->mats;
        const float (*sdir)[3] = MANY ? e->sdir : sh->sdir;
        const float (*sinv)[3] = MANY ? e->sinv : sh->sinv;
        float4* out = MANY ? e->out : one->out;
        const bool rngSin = p.rngMode == 1u;
        const f3 sun = mk(p.sunStrength[0], p.sunStrength[1], p.sunStrength[2]);
        const f3 sunDir = mk(p.sunDir[0], p.sunDir[1], p.sunDir[2]);
        const uint32_t K = p.K;

        packet_setup(W.v[lane], req, lane, m, p, mats, MANY ? e->reqs : one->reqs, MANY ? e->nsamples : one->nsamples, out);
        __syncwarp();
        const uint32_t myFlags = W.v[lane].flags;
        const uint32_t rounds = K <= 32u ? 1u : (K + 31u) / 32u;
        const uint32_t vpp = K <= 32u ? 32u / K : 1u;
        const uint32_t specAll = __ballot_sync(0xFFFFFFFFu, (myFlags & (PV_VALID | PV_SPEC)) == (PV_VALID | PV_SPEC));
        const uint32_t specMask = p.specBounceLimit > 0u ? specAll : 0u;
        // no specular segments: the sum stays zero and is still divided by K
        if (!specMask && ((specAll >> lane) & 1u)) W.v[lane].spec = divs(mk(0.0f, 0.0f, 0.0f), (float)K);
        const uint32_t diffMask = __ballot_sync(0xFFFFFFFFu, (myFlags & (PV_VALID | PV_DIFF)) == (PV_VALID | PV_DIFF));
        const uint32_t firstMask = diffMask & __ballot_sync(0xFFFFFFFFu, (myFlags & PV_FIRST) != 0u);
        const uint32_t fanMask = diffMask & ~firstMask;
        const uint32_t nSpec = (uint32_t)__popc(specMask), nFan = (uint32_t)__popc(fanMask);

        // per-lane state, shared by the passes
        Seg s;
        uint32_t hs = 0, hitIdx = 0;
        bool live = false, stepping = false;
        int vi = -1;                 // voxel of this lane's ray in the current unit
        uint32_t kk = 0, sg = 0;     // ray index, segment of the pack
        f3 pacc = mk(0.0f, 0.0f, 0.0f), cc = pacc;
        uint32_t pi = 0, ncon = 0;
        bool has = false;
        // the ray job's state: specular mult / last position / reflect type / bounce, or diffuse_dir's view of
        // this lane's path (lane == voxel in the diffuse pass)
        Job jd;

        uint32_t pass = PP_SPEC, base = 0, round = 0;
        bool unitOpen = false;
        for (int guard = 0; guard < (1 << 30); guard++) {
            if (!__any_sync(0xFFFFFFFFu, live)) {
                // ---- close the unit: ordered sums
                if (unitOpen) {
                    if (pass == PP_SPEC) {
                        W.ncon[lane] = vi >= 0 ? ncon : 0u;
                        __syncwarp();
                        if (vi >= 0) {
                            const uint32_t nk = K <= 32u ? K : ((K - 32u * round) < 32u ? (K - 32u * round) : 32u);
                            for (uint32_t k2 = 0; k2 < nk; k2++) {
                                const uint32_t src = K <= 32u ? sg * K + k2 : k2;
                                const uint32_t n = W.ncon[src];
                                for (uint32_t jj = 0; jj < n; jj++) {
                                    pacc.x = pacc.x + W.con[src][jj][0];
                                    pacc.y = pacc.y + W.con[src][jj][1];
                                    pacc.z = pacc.z + W.con[src][jj][2];
                                }
                            }
                        }
                        __syncwarp();
                        if (round + 1u == rounds && vi >= 0 && (K > 32u ? lane == 0u : lane == sg * K))
                            W.v[vi].spec = divs(pacc, (float)K);
                    } else if (pass == PP_FIRST) {
                        if ((firstMask >> lane) & 1u) W.v[lane].direct = divs(pacc, 1.0f);
                    } else if (pass == PP_FAN) {
                        const uint32_t hasMask = __ballot_sync(0xFFFFFFFFu, has);
                        const uint32_t nk = K <= 32u ? K : ((K - 32u * round) < 32u ? (K - 32u * round) : 32u);
                        for (uint32_t k2 = 0; k2 < nk; k2++) {
                            const uint32_t src = K <= 32u ? sg * K + k2 : k2;
                            const float x = __shfl_sync(0xFFFFFFFFu, cc.x, src);
                            const float y = __shfl_sync(0xFFFFFFFFu, cc.y, src);
                            const float z = __shfl_sync(0xFFFFFFFFu, cc.z, src);
                            if (vi >= 0 && ((hasMask >> src) & 1u)) { pacc.x = pacc.x + x; pacc.y = pacc.y + y; pacc.z = pacc.z + z; }
                        }
                        if (round + 1u == rounds && vi >= 0 && (K > 32u ? lane == 0u : lane == sg * K))
                            W.v[vi].direct = divs(pacc, (float)K);
                    } else {
                        break;                 // the diffuse unit is the last
                    }
                    __syncwarp();
                    // ---- next unit
                    if (++round >= ((pass == PP_SPEC || pass == PP_FAN) ? rounds : 1u)) {
                        round = 0;
                        base += (pass == PP_SPEC || pass == PP_FAN) ? vpp : 32u;
                    }
                }
                // skip finished or empty passes
                for (;;) {
                    const uint32_t nUnits = pass == PP_SPEC ? nSpec : pass == PP_FIRST ? (firstMask ? 1u : 0u)
                                          : pass == PP_FAN ? nFan : (diffMask ? 1u : 0u);
                    if (pass == PP_DONE || base < ((pass == PP_SPEC || pass == PP_FAN) ? nUnits : nUnits * 32u)) break;
                    pass++;
                    base = 0;
                    round = 0;
                }
                if (pass == PP_DONE) break;
                unitOpen = true;
                // ---- open the unit: one segment per lane
                live = false;
                hs = 0;
                vi = -1;
                if (pass == PP_SPEC || pass == PP_FAN) {
                    vi = pass_voxel(pass == PP_SPEC ? specMask : fanMask, base, K, lane, round, kk, sg);
                    if (round == 0u) pacc = mk(0.0f, 0.0f, 0.0f);
                    has = false;
                    cc = mk(0.0f, 0.0f, 0.0f);
                    if (vi >= 0) {
                        const PacketVoxel& pv = W.v[vi];
                        if (pass == PP_SPEC) {
                            const Material& tm = mats[pv.tmat];
                            jd.jA = pv.talbedo; jd.jB = pv.pos0; jd.jU = tm.reflectType; jd.b = 0; ncon = 0;
                            const f3 P = mk(p.spherePts[kk][0], p.spherePts[kk][1], p.spherePts[kk][2]);
                            const f3 sd = adds(normalize(add(muls(pv.refl, (float)tm.shininess), P)), EPS);
                            seg_begin(s, pv.pos0, sd, rcp3(sd));
                        } else {
                            seg_begin(s, pv.pos0, mk(sdir[kk][0], sdir[kk][1], sdir[kk][2]),
                                      mk(sinv[kk][0], sinv[kk][1], sinv[kk][2]));
                        }
                        c.rays++;
                        live = true;
                    }
                } else if (pass == PP_FIRST) {
                    pacc = mk(0.0f, 0.0f, 0.0f);
                    if ((firstMask >> lane) & 1u) {
                        seg_begin(s, W.v[lane].pos0, mk(sdir[64][0], sdir[64][1], sdir[64][2]),
                                  mk(sinv[64][0], sinv[64][1], sinv[64][2]));
                        c.rays++;
                        live = true;
                    }
                } else {
                    // diffuse: lane = voxel; the first path's first segment (or the paths without segments)
                    pacc = mk(0.0f, 0.0f, 0.0f);
                    if ((diffMask >> lane) & 1u) {
                        const PacketVoxel& pv = W.v[lane];
                        jd.key = pv.key; jd.tnormal = pv.tnormal; jd.tmat = pv.tmat;
                        jd.firstSample = (pv.flags & PV_FIRST) != 0u;
                        pi = 0;
                        live = true;
                        hs = 3u;             // "start the next path" (see the shading below)
                    }
                }
                stepping = live && hs == 0u;
            }
            // ---- step every started segment to its end (the single stepping loop)
            while (__any_sync(0xFFFFFFFFu, stepping)) {
                if (stepping) {
                    const uint32_t rr = seg_step(s, m, mats, p.sunStrength, c, hitIdx);
                    if (rr) { stepping = false; hs = rr; }
                }
            }
            // ---- shade the ended segments
            if (!live || hs == 0u) continue;
            if (pass == PP_SPEC) {
                // specular_ray body after step_map (voxelLighting.comp:98-144)
                const PacketVoxel& pv = W.v[vi];
                bool more = false, add_ = false;
                f3 sc = mk(0.0f, 0.0f, 0.0f);
                if (hs == 1u) {
                    Voxel hv;
                    decompress(m, hitIdx, hv);
                    const i3 hp{f2i(truncf(s.pos.x)), f2i(truncf(s.pos.y)), f2i(truncf(s.pos.z))};
                    if (in_map(m, hp)) {
                        uint8_t* vp = &m.tvis[map_index(m, hp)];
                        if (*vp == 0) *vp = 1;
                    }
                    const f3 d = vabs(sub(vfloor(muls(s.pos, 8.0f)), vfloor(muls(jd.jB, 8.0f))));
                    if (!(dot(d, d) <= 1.0f)) {
                        const Material& hm = mats[hv.material];
                        const f3 hd = muls(hv.diff, 1.0f - hm.specular);
                        add_ = true;
                        if (hm.emissive) {
                            sc.x = ((hv.albedo.x * p.emissiveStrength * s.cmul + s.cadd.x) * jd.jA.x) * pv.talbedo.x;
                            sc.y = ((hv.albedo.y * p.emissiveStrength * s.cmul + s.cadd.y) * jd.jA.y) * pv.talbedo.y;
                            sc.z = ((hv.albedo.z * p.emissiveStrength * s.cmul + s.cadd.z) * jd.jA.z) * pv.talbedo.z;
                        } else {
                            const f3 hc = mul(hd, hv.albedo);
                            sc.x = (hc.x * s.cmul + s.cadd.x) * jd.jA.x;
                            sc.y = (hc.y * s.cmul + s.cadd.y) * jd.jA.y;
                            sc.z = (hc.z * s.cmul + s.cadd.z) * jd.jA.z;
                            if (hm.specular != 0.0f) {
                                jd.jA.x = jd.jA.x * (hv.albedo.x * s.cmul * hm.specular);
                                jd.jA.y = jd.jA.y * (hv.albedo.y * s.cmul * hm.specular);
                                jd.jA.z = jd.jA.z * (hv.albedo.z * s.cmul * hm.specular);
                                jd.jU = hm.reflectType;
                                jd.jB = s.pos;
                                const f3 nd = reflect(s.dir, hv.normal);
                                jd.b++;
                                if (jd.b < p.specBounceLimit) {
                                    const TState keep = s.ts;
                                    seg_begin(s, s.pos, nd, rcp3(nd));
                                    s.ts = keep;   // one ray job: bounces keep the transparency state
                                    c.rays++;
                                    more = true;
                                }
                            }
                        }
                    }
                } else if (dot(s.dir, sunDir) > 0.99f) {
                    add_ = true;
                    sc.x = sun.x * s.cmul + s.cadd.x;
                    sc.y = sun.y * s.cmul + s.cadd.y;
                    sc.z = sun.z * s.cmul + s.cadd.z;
                } else {
                    const f3 sky = (jd.jU == 1u) ? sky_color(mk(p.skyBot[0], p.skyBot[1], p.skyBot[2]),
                                                         mk(p.skyTop[0], p.skyTop[1], p.skyTop[2]), s.dir) : sun;
                    add_ = true;
                    sc.x = (sky.x * s.cmul + s.cadd.x) * jd.jA.x;
                    sc.y = (sky.y * s.cmul + s.cadd.y) * jd.jA.y;
                    sc.z = (sky.z * s.cmul + s.cadd.z) * jd.jA.z;
                }
                if (add_ && ncon < PK_MAX_SPEC_SEGMENTS) {   // at most one per segment; the host checks the limit
                    W.con[lane][ncon][0] = sc.x; W.con[lane][ncon][1] = sc.y; W.con[lane][ncon][2] = sc.z;
                    ncon++;
                }
                hs = 0;
                if (more) stepping = true; else live = false;
            } else if (pass == PP_FIRST || pass == PP_FAN) {
                // shadow_ray: an unoccluded ray adds sunStrength * colorMult + colorAdd
                if (hs == 2u) {
                    cc.x = sun.x * s.cmul + s.cadd.x;
                    cc.y = sun.y * s.cmul + s.cadd.y;
                    cc.z = sun.z * s.cmul + s.cadd.z;
                    has = true;
                    if (pass == PP_FIRST) { pacc.x = pacc.x + cc.x; pacc.y = pacc.y + cc.y; pacc.z = pacc.z + cc.z; }
                }
                hs = 0;
                live = false;
            } else {
                // diffuse_ray body after step_map (voxelLighting.comp:176-201); hs == 3: start the next path
                const PacketVoxel& pv = W.v[lane];
                bool pathDone = hs != 3u;
                if (hs == 1u) {
                    Voxel hv;
                    decompress(m, hitIdx, hv);
                    jd.jB = hv.normal;
                    jd.jU = hv.material;
                    const f3 d = vabs(sub(vfloor(muls(pv.pos0, 8.0f)), vfloor(muls(s.pos, 8.0f))));
                    if (!(dot(d, d) < 1.0f)) {
                        const Material& hm = mats[hv.material];
                        if (hm.emissive) {
                            pacc.x = pacc.x + jd.jA.x * (hv.albedo.x * p.emissiveStrength * s.cmul + s.cadd.x);
                            pacc.y = pacc.y + jd.jA.y * (hv.albedo.y * p.emissiveStrength * s.cmul + s.cadd.y);
                            pacc.z = pacc.z + jd.jA.z * (hv.albedo.z * p.emissiveStrength * s.cmul + s.cadd.z);
                        } else {
                            jd.jA.x = jd.jA.x * (hv.albedo.x * s.cmul + s.cadd.x);
                            jd.jA.y = jd.jA.y * (hv.albedo.y * s.cmul + s.cadd.y);
                            jd.jA.z = jd.jA.z * (hv.albedo.z * s.cmul + s.cadd.z);
                            jd.jC = s.dir;
                            jd.b++;
                            if (jd.b < p.diffuseBounceLimit) {
                                const f3 nd = diffuse_dir(jd, p, mats, rngSin);
                                const TState keep = s.ts;
                                seg_begin(s, s.pos, nd, rcp3(nd));
                                s.ts = keep;
                                c.rays++;
                                pathDone = false;
                                stepping = true;
                            }
                        }
                    }
                } else if (hs == 2u) {
                    const float kd = gmax(dot(s.dir, sunDir), 0.0f);
                    pacc.x = pacc.x + (jd.jA.x * kd * sun.x * s.cmul + s.cadd.x);
                    pacc.y = pacc.y + (jd.jA.y * kd * sun.y * s.cmul + s.cadd.y);
                    pacc.z = pacc.z + (jd.jA.z * kd * sun.z * s.cmul + s.cadd.z);
                }
                if (pathDone) { pacc = add(pacc, pv.direct); pi++; }
                hs = 0;
                if (!stepping) {
                    // the next path of this voxel, if any (paths without segments finish at once)
                    live = false;
                    while (pi < p.numDiffuse) {
                        pacc = add(pacc, mk(p.ambient[0], p.ambient[1], p.ambient[2]));
                        if (p.diffuseBounceLimit == 0u) { pacc = add(pacc, pv.direct); pi++; continue; }
                        jd.i = pi; jd.b = 0;
                        jd.jA = mk(1.0f, 1.0f, 1.0f);
                        jd.jB = adds(jd.tnormal, EPS);
                        jd.jC = mk(0.0f, 0.0f, 0.0f);
                        jd.jU = jd.tmat;
                        const f3 nd = diffuse_dir(jd, p, mats, rngSin);
                        seg_begin(s, pv.pos0, nd, rcp3(nd));
                        c.rays++;
                        live = true;
                        stepping = true;
                        break;
                    }
                }
            }
        }
        // ---- write the voxel's new lighting (voxelLighting.comp:266-288, FP32)
        __syncwarp();
        if (myFlags & PV_VALID) {
            const PacketVoxel& pv = W.v[lane];
            f3 dacc = mk(0.0f, 0.0f, 0.0f);
            if (myFlags & PV_DIFF) {
                const float4 prev = __ldg(&m.diff[pv.vidx]);
                const float den = pv.indirect + (float)p.numDiffuse;
                dacc.x = (prev.x * pv.indirect + pacc.x) / den;
                dacc.y = (prev.y * pv.indirect + pacc.y) / den;
                dacc.z = (prev.z * pv.indirect + pacc.z) / den;
            }
            const f3 sp = (myFlags & PV_SPEC) ? pv.spec : mk(0.0f, 0.0f, 0.0f);
            const float4 outS = make_float4(gmin(gmax(sp.x, 0.0f), 1.0f), gmin(gmax(sp.y, 0.0f), 1.0f),
                                            gmin(gmax(sp.z, 0.0f), 1.0f), 0.0f);
            const float4 outD = make_float4(gmin(gmax(dacc.x, 0.0f), 1.0f), gmin(gmax(dacc.y, 0.0f), 1.0f),
                                            gmin(gmax(dacc.z, 0.0f), 1.0f), 0.0f);
            const uint64_t o = ((uint64_t)req * 32u + lane) * 2u;
            out[o] = outD;
            out[o + 1] = outS;
            lit++;
        }
        __syncwarp();
    }
    flush_counters(MANY ? many->stats : one->stats, c, 0, lit);
}

} // namespace dn
