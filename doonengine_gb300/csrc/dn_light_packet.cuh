/*
 * dn_light_packet.cuh -- the lighting update with ray fans traced as warp packets.
 *
 * Every lit voxel casts two fans of K rays from one point: K specular rays around its reflection
 * direction (voxelLighting.comp:83-146, each up to specBounceLimit segments) and K shadow rays around the
 * sun direction (D8).  A warp takes one work unit -- 32 / PK_PARTS voxels of a request group (a group is 32
 * voxels of one chunk) in a one-map launch, a whole group in a many-map launch -- and traces the fans of
 * PK_POOL_FAN / K of its voxels at a time as one pool: the pool's rays are numbered (specular fans first,
 * then the shadow rays), and a lane whose ray has ended takes the pool's next ray, so consecutive rays of
 * a fan run side by side and the lanes of a warp walk nearly the same cells (a fan's shadow rays are
 * almost parallel, its specular rays share their origin and lobe).  Ended segments are shaded once
 * `batch` lanes have one.  Each ray's contributions go to shared memory; when the pool is empty, each
 * voxel's sums are formed by one lane walking its rays (and their segments) in ray order, so every sum
 * is accumulated in exactly the reference's order.  The kernel writes each voxel's specular lighting and
 * leaves its direct light for the diffuse kernel (dn_light_stream.cuh, stream_loop<.., true>), which traces
 * the diffuse paths (numDiffuse per voxel, up to diffuseBounceLimit segments each) as per-lane path
 * streams over all request groups and finishes each voxel as the reference's lighting main does (running
 * average, clamps, voxelLighting.comp:238-288).
 *
 * Results, traversal side effects (requested / touched / visible flags) and counters are those of the
 * one-voxel-per-lane form (dn_light_stream.cuh): the same rays are traced with the same
 * operations; only the assignment of rays to lanes differs.
 */
#pragma once
#include "dn_light_stream.cuh"

namespace dn {

#ifndef DN_PACKET_MIN_BLOCKS
#define DN_PACKET_MIN_BLOCKS 6   // 6 blocks of 4 warps per SM (measured best on the large map: 5 and 4 are slower)
#endif

// specBounceLimit handled here (the reference's default is 2); larger limits use the stream kernel
constexpr uint32_t PK_MAX_SPEC_SEGMENTS = 2;

// per-voxel data of the warp's request group (shared memory, written by the voxel's lane)
struct PacketVoxel {
    f3 pos0, tnormal, talbedo, refl;
    f3 spec;                 // specular sum / K (after the specular pass)
    f3 direct;               // shadow sum / n (after the shadow pass)
    uint32_t tmat, key, vidx, flags;   // flags: 1 valid, 2 first sample, 4 specular pass, 8 diffuse passes
    float indirect;
};
enum : uint32_t { PV_VALID = 1u, PV_FIRST = 2u, PV_SPEC = 4u, PV_DIFF = 8u };

// rays per fan kind in one pool (voxels per pool = PK_POOL_FAN / K): the pool's specular contributions,
// shadow contributions and counts live in shared memory, 38 B per pooled ray.  Larger pools shorten the
// tail that a pool's longest rays leave; the shared memory they take comes out of L1 (the SM's 256 KB
// split).  Measured on the large map at 6 blocks per SM with the tables in global memory: 64 rays
// 3.38 G rays/s, 96 3.55, 128 3.64-3.66 (31 KB per block, 60 KB of L1), 160 3.60, 192 (5 blocks) 3.40.
#ifndef DN_PK_POOL_FAN
#define DN_PK_POOL_FAN 128
#endif
constexpr uint32_t PK_POOL_FAN = DN_PK_POOL_FAN;
constexpr uint32_t PK_POOL_ALT = PK_POOL_FAN == 64u ? 128u : 64u;   // the batched autotuner's other pool size

// Work units per request group in a one-map launch: a warp takes 32 / PK_PARTS voxels of a group at a time,
// so that the launch does not end with a few warps finishing whole groups while the others have left.  Per
// warp exit times on the large map's frame 11 with whole groups: the last warp left 2.7 ms after 90 % of
// them had, 16 % of the warps' time idle; units of 16, 8 and 4 voxels measured +8 %, +12 % and +13 %.  A
// many-map launch keeps whole groups: its queue is long enough that the tail is small, and smaller units
// measured slower there (the setup of a unit runs on a fraction of the lanes).
#ifndef DN_PK_PARTS
#define DN_PK_PARTS 8
#endif
constexpr uint32_t PK_PARTS = DN_PK_PARTS;
static_assert(PK_PARTS == 1u || PK_PARTS == 2u || PK_PARTS == 4u || PK_PARTS == 8u,
              "a unit is 32, 16, 8 or 4 voxels of a group");

template <uint32_t POOL>
struct PacketWarpT {
    PacketVoxel v[32];
    float con[POOL][PK_MAX_SPEC_SEGMENTS][3];   // specular contributions of each pooled ray, in segment order
    float sh[POOL][3];                          // shadow contribution of each pooled ray
    uint8_t ncon[POOL];                         // contributions of each specular ray
    uint8_t shHas[POOL];                        // the shadow ray was unoccluded
};
using PacketWarp = PacketWarpT<PK_POOL_FAN>;

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

// The work units of one launch (a part of a request group, or a whole group in a many-map launch).  Per
// unit: (1) pools of PK_POOL_FAN/K voxels (at least one): every ray of their specular fans, first-sample
// shadow rays and shadow fans is traced by whichever lane is free -- a lane takes the pool's next ray as
// soon as its own ended, and the shading of ended segments runs once `batch` lanes have one, so no lane
// waits for the slowest ray of a fan; each ray's contributions go to shared memory, and when the pool is
// empty every voxel's sums are formed in the reference's order; (2) the write-out of each voxel's
// specular lighting and direct light (its diffuse paths run in k_light_diffuse).
template <bool MANY, uint32_t POOL = PK_POOL_FAN>
__device__ __forceinline__ void packet_loop(const StreamArgs* one, const BatchLightArgs* many, PacketWarpT<POOL>& W)
{
    const uint32_t lane = lane_id_s();
    uint32_t nreq = 0;
    if constexpr (MANY) nreq = *(volatile const uint32_t*)&many->reqStart[many->nmaps];
    else nreq = *(volatile const uint32_t*)one->nreqPtr;
    uint32_t* const counter = MANY ? many->workCounter : one->workCounter;
    const uint32_t batch = MANY ? many->batch : one->batch;
    Counters c{0, 0, 0, 0, 0};
    uint32_t lit = 0;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(counter, 1u);
        u = __shfl_sync(0xFFFFFFFFu, u, 0);
        constexpr uint32_t parts = MANY ? 1u : PK_PARTS;
        if (u >= nreq * parts) break;
        // unit u: lanes [part * 32 / parts, (part + 1) * 32 / parts) of request group r
        const uint32_t r = u / parts;
        const bool mine = lane / (32u / parts) == u % parts;
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
        const Material* mats = MANY ? e->mats : one->gtab->mats;
        const float (*sdir)[3] = MANY ? e->sdir : one->gtab->sdir;
        const float (*sinv)[3] = MANY ? e->sinv : one->gtab->sinv;
        float4* out = MANY ? e->out : one->out;
        const f3 sun = mk(p.sunStrength[0], p.sunStrength[1], p.sunStrength[2]);
        const f3 sunDir = mk(p.sunDir[0], p.sunDir[1], p.sunDir[2]);
        const uint32_t K = p.K;

        if (mine) packet_setup(W.v[lane], req, lane, m, p, mats, MANY ? e->reqs : one->reqs, MANY ? e->nsamples : one->nsamples, out);
        else W.v[lane].flags = 0;   // another unit's voxel: its warp sets it up and writes it
        __syncwarp();
        const uint32_t myFlags = W.v[lane].flags;
        const uint32_t specAll = __ballot_sync(0xFFFFFFFFu, (myFlags & (PV_VALID | PV_SPEC)) == (PV_VALID | PV_SPEC));
        const uint32_t specMask = p.specBounceLimit > 0u ? specAll : 0u;
        // no specular segments: the sum stays zero and is still divided by K
        if (!specMask && ((specAll >> lane) & 1u)) W.v[lane].spec = divs(mk(0.0f, 0.0f, 0.0f), (float)K);
        const uint32_t diffMask = __ballot_sync(0xFFFFFFFFu, (myFlags & (PV_VALID | PV_DIFF)) == (PV_VALID | PV_DIFF));
        const uint32_t firstMask = diffMask & __ballot_sync(0xFFFFFFFFu, (myFlags & PV_FIRST) != 0u);
        const uint32_t workMask = specMask | diffMask;
        const uint32_t nWork = (uint32_t)__popc(workMask);
        const uint32_t perPool = K < POOL ? POOL / K : 1u;

        // per-lane ray state
        Seg s;
        uint32_t hs = 0, hitIdx = 0;
        bool live = false, stepping = false;
        uint32_t rid = 0, ncon = 0;       // the lane's ray: index in its fan array; contributions so far
        bool isSpec = false;
        int vi = -1;                      // the ray's voxel
        Job jd;                           // specular: jA mult, jB last position, jU reflect type, b bounce

        // ---- (1) pools of specular and shadow fans
        for (uint32_t base = 0; base < nWork; base += perPool) {
            // the pool's voxels: slots j < np of workMask, from bit 'base' on; ray layout:
            // [specular rays of voxel 0, 1, ...] then [shadow rays of voxel 0, 1, ...]
            uint32_t rest = workMask;
            for (uint32_t t = 0; t < base; t++) rest &= rest - 1u;
            const uint32_t np = (nWork - base) < perPool ? (nWork - base) : perPool;
            uint32_t poolMask = 0, rm = rest;
            for (uint32_t t = 0; t < np; t++) { poolMask |= rm & (0u - rm); rm &= rm - 1u; }
            const uint32_t nSpecRays = (uint32_t)__popc(poolMask & specMask) * K;
            const uint32_t nFanVox = (uint32_t)__popc(poolMask & diffMask & ~firstMask);
            const uint32_t nFirst = (uint32_t)__popc(poolMask & firstMask);
            const uint32_t nShRays = nFanVox * K + nFirst;   // shadow rays in voxel order (1 or K per voxel)
            const uint32_t total = nSpecRays + nShRays;
            uint32_t next = 0;
            for (int guard = 0; guard < (1 << 30); guard++) {
                // lanes without a ray take the pool's next rays in order
                const unsigned need = __ballot_sync(0xFFFFFFFFu, !live);
                if (next < total && need) {
                    const uint32_t rank = __popc(need & ((1u << lane) - 1u));
                    if (!live && next + rank < total) {
                        const uint32_t q = next + rank;
                        if (q < nSpecRays) {
                            // specular ray kk of the pool's (q / K)-th specular voxel
                            isSpec = true;
                            rid = q;
                            const uint32_t kk = q % K;
                            uint32_t mm = poolMask & specMask;
                            for (uint32_t t = 0; t < q / K; t++) mm &= mm - 1u;
                            vi = __ffs(mm) - 1;
                            const PacketVoxel& pv = W.v[vi];
                            const Material& tm = mats[pv.tmat];
                            jd.jA = pv.talbedo; jd.jB = pv.pos0; jd.jU = tm.reflectType; jd.b = 0; ncon = 0;
                            const f3 P = mk(p.spherePts[kk][0], p.spherePts[kk][1], p.spherePts[kk][2]);
                            const f3 sd = adds(normalize(add(muls(pv.refl, (float)tm.shininess), P)), EPS);
                            seg_begin(s, pv.pos0, sd, rcp3(sd));
                        } else {
                            // shadow ray: voxels of the pool in slot order, K rays each (1 on the first sample)
                            isSpec = false;
                            rid = q - nSpecRays;
                            uint32_t mm = poolMask & diffMask, off = 0, kk = 0;
                            vi = -1;
                            while (mm) {
                                const int v = __ffs(mm) - 1;
                                mm &= mm - 1u;
                                const uint32_t n = ((firstMask >> v) & 1u) ? 1u : K;
                                if (rid < off + n) { vi = v; kk = ((firstMask >> v) & 1u) ? 64u : rid - off; break; }
                                off += n;
                            }
                            seg_begin(s, W.v[vi].pos0, mk(sdir[kk][0], sdir[kk][1], sdir[kk][2]),
                                      mk(sinv[kk][0], sinv[kk][1], sinv[kk][2]));
                        }
                        c.rays++;
                        live = true;
                        stepping = true;
                        hs = 0;
                    }
                    next = (next + (uint32_t)__popc(need)) < total ? next + (uint32_t)__popc(need) : total;
                }
                const unsigned liveMask = __ballot_sync(0xFFFFFFFFu, live);
                if (!liveMask) break;
                // step until 'batch' lanes have an ended segment (or none is left stepping); the live lanes
                // do not change while stepping, so one vote per step tells both
                for (;;) {
                    const unsigned st = __ballot_sync(0xFFFFFFFFu, stepping);
                    if (!st || (uint32_t)__popc(liveMask & ~st) >= batch) break;
                    if (stepping) {
                        const uint32_t rr = seg_step(s, m, mats, p.sunStrength, c, hitIdx);
                        if (rr) { stepping = false; hs = rr; }
                    }
                }
                // shade the ended segments
                if (!live || stepping) continue;
                if (isSpec) {
                    // specular_ray body after step_map (voxelLighting.comp:98-144)
                    const PacketVoxel& pv = W.v[vi];
                    bool more = false, add_ = false;
                    f3 sc = mk(0.0f, 0.0f, 0.0f);
                    if (hs == 1u) {
                        hit_position(s);
                        Voxel hv;
                        decompress(m, hit_index(s, hitIdx), hv);
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
                        W.con[rid][ncon][0] = sc.x; W.con[rid][ncon][1] = sc.y; W.con[rid][ncon][2] = sc.z;
                        ncon++;
                    }
                    hs = 0;
                    if (more) stepping = true;
                    else { W.ncon[rid] = (uint8_t)ncon; live = false; }
                } else {
                    // shadow_ray: an unoccluded ray adds sunStrength * colorMult + colorAdd
                    const bool miss = hs == 2u;
                    W.sh[rid][0] = sun.x * s.cmul + s.cadd.x;
                    W.sh[rid][1] = sun.y * s.cmul + s.cadd.y;
                    W.sh[rid][2] = sun.z * s.cmul + s.cadd.z;
                    W.shHas[rid] = miss ? 1 : 0;
                    hs = 0;
                    live = false;
                }
            }
            __syncwarp();
            // the pool's sums in the reference's order: lane 2j sums voxel j's specular rays (ray, then
            // segment order), lane 2j+1 its shadow rays; pools of more than 16 voxels (small K) take a
            // second round
            for (uint32_t j = lane >> 1; j < np; j += 16u) {
                {
                    uint32_t mm = poolMask;
                    for (uint32_t t = 0; t < j; t++) mm &= mm - 1u;
                    const int v = __ffs(mm) - 1;
                    f3 acc = mk(0.0f, 0.0f, 0.0f);
                    if ((lane & 1u) == 0u) {
                        if ((specMask >> v) & 1u) {
                            const uint32_t r0 = (uint32_t)__popc(poolMask & specMask & ((1u << v) - 1u)) * K;
                            for (uint32_t k2 = 0; k2 < K; k2++) {
                                const uint32_t n = W.ncon[r0 + k2];
                                for (uint32_t jj = 0; jj < n; jj++) {
                                    acc.x = acc.x + W.con[r0 + k2][jj][0];
                                    acc.y = acc.y + W.con[r0 + k2][jj][1];
                                    acc.z = acc.z + W.con[r0 + k2][jj][2];
                                }
                            }
                            W.v[v].spec = divs(acc, (float)K);
                        }
                    } else if ((diffMask >> v) & 1u) {
                        uint32_t r0 = 0, mm2 = poolMask & diffMask & ((1u << v) - 1u);
                        while (mm2) {
                            const int u = __ffs(mm2) - 1;
                            mm2 &= mm2 - 1u;
                            r0 += ((firstMask >> u) & 1u) ? 1u : K;
                        }
                        const uint32_t n = ((firstMask >> v) & 1u) ? 1u : K;
                        for (uint32_t k2 = 0; k2 < n; k2++)
                            if (W.shHas[r0 + k2]) {
                                acc.x = acc.x + W.sh[r0 + k2][0];
                                acc.y = acc.y + W.sh[r0 + k2][1];
                                acc.z = acc.z + W.sh[r0 + k2][2];
                            }
                        W.v[v].direct = divs(acc, (float)n);
                    }
                }
            }
            __syncwarp();
        }

        // ---- (2) write the voxel's specular lighting (voxelLighting.comp:266-288, FP32).  Its diffuse paths
        // run in the diffuse kernel that follows (k_light_diffuse: per-lane path streams, so that one long
        // path does not hold the other 31 lanes), which reads the direct light left here in the diffuse slot
        // and replaces it with the voxel's new diffuse lighting; a voxel without diffuse paths gets zero.
        __syncwarp();
        if (myFlags & PV_VALID) {
            const PacketVoxel& pv = W.v[lane];
            const f3 sp = (myFlags & PV_SPEC) ? pv.spec : mk(0.0f, 0.0f, 0.0f);
            const float4 outS = make_float4(gmin(gmax(sp.x, 0.0f), 1.0f), gmin(gmax(sp.y, 0.0f), 1.0f),
                                            gmin(gmax(sp.z, 0.0f), 1.0f), 0.0f);
            const float4 outD = (myFlags & PV_DIFF) ? make_float4(pv.direct.x, pv.direct.y, pv.direct.z, 0.0f)
                                                    : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
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
