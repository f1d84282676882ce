/*
 * dn_light.cuh -- lighting rays on the device (voxelLighting.comp:65-288).
 *
 * trace_light() is the two-level DDA of voxelShared.comp:328-475 for lighting
 * rays (refraction off, maxDepth < 0, first voxel ignored) written as ONE loop:
 * each iteration is either one chunk-cell step or one voxel step.  The nested
 * reference form (an outer chunk loop that calls an inner voxel loop) keeps
 * lanes of a warp in different loops and serialises them; the flattened form
 * keeps every lane in the same loop body.  It performs the same floating-point
 * operations in the same order as the nested form, so it visits the same
 * cells and hits the same voxels bit for bit.  The hit normal the nested form
 * tracks is only read by refraction, which lighting disables, so it is not
 * computed here.
 */
#pragma once
#include "dn_device.cuh"

namespace dn {

// one lighting ray segment: step_map(dir, 1/dir, rayPos, true, -1, tmp, hv, cadd, cmul) with refraction off
__device__ __forceinline__ bool trace_light(RayCtx& c, TState& ts, const f3 dir, f3& rayPos, Voxel& hv, f3& cadd,
                                            float& cmul)
{
    const DevMap& m = *c.m;
    const f3 inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    bool requested = false;
    cadd = mk(0.0f, 0.0f, 0.0f);
    cmul = 1.0f;
    c.c.rays++;
    i3 opos, step; f3 delta, oside;
    init_dda(dir, inv, rayPos, opos, delta, step, oside);
    f3 olast = mk(0.0f, 0.0f, 0.0f);
    bool oIgnore = true;
    // inner level state
    bool inner = false, iIgnore = false;
    i3 ipos = {0, 0, 0};
    f3 iside = olast, ilast = olast, cp = olast;
    const ChunkRec* rec = nullptr;
    uint32_t base = 0;
    while (true) {
        if (!inner) {
            if (!in_map(m, opos)) return false;
            c.c.outer++;
            const uint32_t t = map_index(m, opos);
            const uint32_t w = __ldg(&m.tword[t]);
            const uint32_t st = w >> 30;
            if (st == 2u) {
                c.c.entered++;
                if (m.ttouch[t] == 0) m.ttouch[t] = 1;
                const float tt = min3(olast) - EPS;
                const f3 up = add(rayPos, muls(dir, tt));
                cp = mk((up.x - (float)opos.x) * 8.0f, (up.y - (float)opos.y) * 8.0f, (up.z - (float)opos.z) * 8.0f);
                const float lo = EPS, hi_ = 8.0f - EPS;
                cp.x = gmin(gmax(cp.x, lo), hi_); cp.y = gmin(gmax(cp.y, lo), hi_); cp.z = gmin(gmax(cp.z, lo), hi_);
                // init_DDA at the chunk-local position (delta and step are those of the outer level: same direction)
                const f3 fl = vfloor(cp);
                ipos.x = f2i(fl.x); ipos.y = f2i(fl.y); ipos.z = f2i(fl.z);
                const f3 s = mk((float)step.x, (float)step.y, (float)step.z);
                iside.x = (s.x * ((float)ipos.x - cp.x) + s.x * 0.5f + 0.5f) * delta.x;
                iside.y = (s.y * ((float)ipos.y - cp.y) + s.y * 0.5f + 0.5f) * delta.y;
                iside.z = (s.z * ((float)ipos.z - cp.z) + s.z * 0.5f + 0.5f) * delta.z;
                ilast = mk(0.0f, 0.0f, 0.0f);
                iIgnore = oIgnore;
                rec = &m.rec[w & SLOT_MASK];
                base = __ldg(&rec->voxBase);
                inner = true;
                continue;
            } else if (!requested && st != 0u) {
                if (m.treq[t] == 0) m.treq[t] = 1;
                requested = true;
            }
            olast = oside;
            {
                const bool mx = oside.x <= gmin(oside.y, oside.z);
                const bool my = oside.y <= gmin(oside.z, oside.x);
                const bool mz = oside.z <= gmin(oside.x, oside.y);
                oside.x = oside.x + (mx ? 1.0f : 0.0f) * delta.x;
                oside.y = oside.y + (my ? 1.0f : 0.0f) * delta.y;
                oside.z = oside.z + (mz ? 1.0f : 0.0f) * delta.z;
                opos.x += (int32_t)mx * step.x; opos.y += (int32_t)my * step.y; opos.z += (int32_t)mz * step.z;
            }
            oIgnore = false;
            continue;
        }
        if (!in_chunk(ipos)) {
            // the chunk was crossed without a hit: the outer loop iterates
            inner = false;
            olast = oside;
            const bool mx = oside.x <= gmin(oside.y, oside.z);
            const bool my = oside.y <= gmin(oside.z, oside.x);
            const bool mz = oside.z <= gmin(oside.x, oside.y);
            oside.x = oside.x + (mx ? 1.0f : 0.0f) * delta.x;
            oside.y = oside.y + (my ? 1.0f : 0.0f) * delta.y;
            oside.z = oside.z + (mz ? 1.0f : 0.0f) * delta.z;
            opos.x += (int32_t)mx * step.x; opos.y += (int32_t)my * step.y; opos.z += (int32_t)mz * step.z;
            oIgnore = false;
            continue;
        }
        c.c.inner++;
        const uint32_t li = (uint32_t)(ipos.x + 8 * (ipos.y + 8 * ipos.z));
        const bool exists = (__ldg(&rec->mask[li >> 5]) >> (li & 31)) & 1u;
        if (exists && !iIgnore) {
            const uint32_t idx = base + vox_rank(rec, li);
            c.c.hits++;
            const uint2 w = __ldg(&m.vox[idx]);
            const uint32_t material = w.x >> 24;
            const Material& mat = c.mats[material];
            if (mat.opacity == 1.0f) {
                const float t = min3(ilast) + EPS;
                cp = add(cp, muls(dir, t));
                decompress(m, idx, hv);
                rayPos = add(mk((float)opos.x, (float)opos.y, (float)opos.z), muls(cp, INV_CHUNK));
                return true;
            }
            const uint32_t thisID = (w.y & 0xFFFFFF00u) | material;
            if (ts.lastVoxID != thisID) {
                const f3 alb = mk((float)((w.y >> 24) & 0xFF) * INV255, (float)((w.y >> 16) & 0xFF) * INV255,
                                  (float)((w.y >> 8) & 0xFF) * INV255);
                const float k = cmul * mat.opacity;
                cadd.x = cadd.x + k * alb.x * c.sunStrength.x;
                cadd.y = cadd.y + k * alb.y * c.sunStrength.y;
                cadd.z = cadd.z + k * alb.z * c.sunStrength.z;
                cmul = cmul * (1.0f - mat.opacity);
                ts.lastVoxID = thisID;
                ts.lastVoxRefract = mat.refractIndex;
            }
        } else if (ts.lastVoxID != 255u) {
            ts.lastVoxID = 255u;
            ts.lastVoxRefract = 1.0f;
        }
        ilast = iside;
        {
            const bool mx = iside.x <= gmin(iside.y, iside.z);
            const bool my = iside.y <= gmin(iside.z, iside.x);
            const bool mz = iside.z <= gmin(iside.x, iside.y);
            iside.x = iside.x + (mx ? 1.0f : 0.0f) * delta.x;
            iside.y = iside.y + (my ? 1.0f : 0.0f) * delta.y;
            iside.z = iside.z + (mz ? 1.0f : 0.0f) * delta.z;
            ipos.x += (int32_t)mx * step.x; ipos.y += (int32_t)my * step.y; ipos.z += (int32_t)mz * step.z;
        }
        iIgnore = false;
    }
}

struct LightCtx {
    RayCtx rc;
    const dn_light_params* p;
    f3 sunDir, ambient, camPos, skyBot, skyTop;
    bool firstSample, rngSin;
    uint32_t key, sample;
};

// specular_ray, voxelLighting.comp:83-146
__device__ __forceinline__ void specular_ray(LightCtx& L, f3 rayPos, f3 rayDir, f3 albedo, uint32_t reflectType, f3& color)
{
    RayCtx& c = L.rc;
    const DevMap& m = *c.m;
    f3 lastPos = rayPos;
    f3 mult = albedo;
    Voxel hv;
    TState ts{255u, 1.0f};   // D13: fresh per ray job
    for (uint32_t i = 0; i < L.p->specBounceLimit; i++) {
        f3 cadd; float cmul;
        if (trace_light(c, ts, rayDir, rayPos, hv, cadd, cmul)) {
            const i3 hp{f2i(truncf(rayPos.x)), f2i(truncf(rayPos.y)), f2i(truncf(rayPos.z))};
            if (in_map(m, hp)) {   // D4: the lit chunk was visible when requested
                uint8_t* vp = &m.tvis[map_index(m, hp)];
                if (*vp == 0) *vp = 1;
            }
            const f3 d = vabs(sub(vfloor(muls(rayPos, 8.0f)), vfloor(muls(lastPos, 8.0f))));
            if (dot(d, d) <= 1.0f) return;
            const Material& hm = c.mats[hv.material];
            hv.diff = muls(hv.diff, 1.0f - hm.specular);
            if (hm.emissive) {
                color.x = color.x + ((hv.albedo.x * c.emissive * cmul + cadd.x) * mult.x) * albedo.x;
                color.y = color.y + ((hv.albedo.y * c.emissive * cmul + cadd.y) * mult.y) * albedo.y;
                color.z = color.z + ((hv.albedo.z * c.emissive * cmul + cadd.z) * mult.z) * albedo.z;
                return;
            }
            const f3 hc = mul(hv.diff, hv.albedo);
            color.x = color.x + (hc.x * cmul + cadd.x) * mult.x;
            color.y = color.y + (hc.y * cmul + cadd.y) * mult.y;
            color.z = color.z + (hc.z * cmul + cadd.z) * mult.z;
            if (hm.specular == 0.0f) return;
            mult.x = mult.x * (hv.albedo.x * cmul * hm.specular);
            mult.y = mult.y * (hv.albedo.y * cmul * hm.specular);
            mult.z = mult.z * (hv.albedo.z * cmul * hm.specular);
            reflectType = hm.reflectType;
            lastPos = rayPos;
            rayDir = reflect(rayDir, hv.normal);
        } else if (dot(rayDir, L.sunDir) > 0.99f) {
            color.x = color.x + (c.sunStrength.x * cmul + cadd.x);
            color.y = color.y + (c.sunStrength.y * cmul + cadd.y);
            color.z = color.z + (c.sunStrength.z * cmul + cadd.z);
            return;
        } else {
            const f3 s = (reflectType == 1u) ? sky_color(L.skyBot, L.skyTop, rayDir) : c.sunStrength;
            color.x = color.x + (s.x * cmul + cadd.x) * mult.x;
            color.y = color.y + (s.y * cmul + cadd.y) * mult.y;
            color.z = color.z + (s.z * cmul + cadd.z) * mult.z;
            return;
        }
    }
}

// diffuse_ray, voxelLighting.comp:149-203
__device__ __forceinline__ void diffuse_ray(LightCtx& L, f3 normal, f3 rayPos, const Voxel& initial, float seed, f3& color)
{
    RayCtx& c = L.rc;
    const dn_light_params* p = L.p;
    Voxel hv = initial;
    f3 hitNormal = normal;
    uint32_t hmat = initial.material;
    f3 nc = mk(1.0f, 1.0f, 1.0f);
    const f3 lastPos = rayPos;
    f3 lastDir = mk(0.0f, 0.0f, 0.0f);
    TState ts{255u, 1.0f};   // D13
    for (uint32_t i = 0; i < p->diffuseBounceLimit; i++) {
        f3 dir;
        bool lobe = false;
        const Material& hm0 = c.mats[hmat];
        if (i > 0) {
            const float r = L.rngSin ? srand1(seed + (float)p->diffuseBounceLimit + (float)i)
                                     : hrand(L.key, 2u, (L.sample * 16u + i) << 8);
            lobe = (r + 1.0f) * 0.5f < hm0.specular;
        }
        if (lobe) {
            const f3 rs = L.rngSin ? sphere_sin(p->time + (float)i) : sphere_hash(L.key, 3u, L.sample * 16u + i);
            dir = normalize(add(muls(reflect(lastDir, hitNormal), (float)hm0.shininess), rs));
        } else if (L.firstSample) {
            dir = adds(normalize(hitNormal), EPS);
        } else {
            const f3 rs = L.rngSin ? sphere_sin(seed + (float)i) : sphere_hash(L.key, 1u, L.sample * 16u + i);
            dir = adds(normalize(add(hitNormal, rs)), EPS);
        }
        f3 cadd; float cmul;
        const bool hit = trace_light(c, ts, dir, rayPos, hv, cadd, cmul);
        hitNormal = hv.normal;
        hmat = hv.material;
        const Material& hm = c.mats[hmat];
        if (hit) {
            const f3 d = vabs(sub(vfloor(muls(lastPos, 8.0f)), vfloor(muls(rayPos, 8.0f))));
            if (dot(d, d) < 1.0f) return;
            if (hm.emissive) {
                color.x = color.x + nc.x * (hv.albedo.x * c.emissive * cmul + cadd.x);
                color.y = color.y + nc.y * (hv.albedo.y * c.emissive * cmul + cadd.y);
                color.z = color.z + nc.z * (hv.albedo.z * c.emissive * cmul + cadd.z);
                return;
            }
            nc.x = nc.x * (hv.albedo.x * cmul + cadd.x);
            nc.y = nc.y * (hv.albedo.y * cmul + cadd.y);
            nc.z = nc.z * (hv.albedo.z * cmul + cadd.z);
        } else {
            const float k = gmax(dot(dir, L.sunDir), 0.0f);
            color.x = color.x + (nc.x * k * c.sunStrength.x * cmul + cadd.x);
            color.y = color.y + (nc.y * k * c.sunStrength.y * cmul + cadd.y);
            color.z = color.z + (nc.z * k * c.sunStrength.z * cmul + cadd.z);
            return;
        }
        lastDir = dir;
    }
}

// one shadow ray, voxelLighting.comp:65-80
__device__ __forceinline__ void shadow_ray(LightCtx& L, f3 rayPos, f3 dir, f3& color)
{
    RayCtx& c = L.rc;
    Voxel hv; f3 cadd; float cmul;
    TState ts{255u, 1.0f};   // D13
    if (!trace_light(c, ts, dir, rayPos, hv, cadd, cmul)) {
        color.x = color.x + (c.sunStrength.x * cmul + cadd.x);
        color.y = color.y + (c.sunStrength.y * cmul + cadd.y);
        color.z = color.z + (c.sunStrength.z * cmul + cadd.z);
    }
}

// voxelLighting.comp:207-288 for one voxel.  Every lane of a warp lights a voxel of the same chunk and
// walks the same ray index k in the same phase, so the K shadow rays of a warp share one direction.
__device__ __forceinline__ void light_voxel(LightCtx& L, bool active, i3 mp, i3 cp, const Voxel& tv, uint32_t samples,
                                            float4& outD, float4& outS)
{
    RayCtx& c = L.rc;
    const DevMap& m = *c.m;
    const dn_light_params* p = L.p;
    const Material& tm = c.mats[tv.material];
    const uint32_t ns = samples < p->maxDiffuse ? samples : p->maxDiffuse;
    const float indirect = (float)ns;
    L.firstSample = (indirect == 0.0f);
    const uint32_t gx = (uint32_t)(mp.x * 8 + cp.x), gy = (uint32_t)(mp.y * 8 + cp.y), gz = (uint32_t)(mp.z * 8 + cp.z);
    const uint32_t gidx = gx + (m.sx * 8u) * (gy + (m.sy * 8u) * gz);
    L.key = rng_key(__float_as_uint(p->time), p->mapId, gidx);

    f3 rayPos;
    rayPos.x = INV_CHUNK * (float)cp.x + (float)mp.x + HALF_INV_CHUNK;
    rayPos.y = INV_CHUNK * (float)cp.y + (float)mp.y + HALF_INV_CHUNK;
    rayPos.z = INV_CHUNK * (float)cp.z + (float)mp.z + HALF_INV_CHUNK;
    const float off = HALF_INV_CHUNK - EPS;
    rayPos = add(rayPos, muls(tv.normal, off));

    f3 spec = mk(0.0f, 0.0f, 0.0f), diff = mk(0.0f, 0.0f, 0.0f);
    const uint32_t K = p->K;
    const f3 viewDir = sub(rayPos, L.camPos);
    const bool doSpec = active && tm.specular > 0.0f && dot(viewDir, tv.normal) < 0.0f && tm.reflectType <= 1u;
    if (__any_sync(0xFFFFFFFFu, doSpec)) {
        const f3 refl = reflect(normalize(viewDir), tv.normal);
        for (uint32_t k = 0; k < K; k++) {
            if (doSpec) {
                const f3 P = mk(p->spherePts[k][0], p->spherePts[k][1], p->spherePts[k][2]);
                const f3 sd = adds(normalize(add(muls(refl, (float)tm.shininess), P)), EPS);
                specular_ray(L, rayPos, sd, tv.albedo, tm.reflectType, spec);
            }
        }
        spec = divs(spec, (float)K);
    }
    const bool doDiff = active && tm.specular < 1.0f;
    if (__any_sync(0xFFFFFFFFu, doDiff)) {
        // D8: K fixed shadow rays traced once, averaged, added once per sample
        f3 sum = mk(0.0f, 0.0f, 0.0f);
        f3 direct;
        if (L.firstSample) {
            if (doDiff) shadow_ray(L, rayPos, adds(L.sunDir, EPS), sum);
            direct = divs(sum, 1.0f);
        } else {
            for (uint32_t k = 0; k < K; k++) {
                if (doDiff) {
                    const f3 P = mk(p->spherePts[k][0], p->spherePts[k][1], p->spherePts[k][2]);
                    const f3 d = adds(normalize(add(muls(L.sunDir, p->shadowSoftness), P)), EPS);
                    shadow_ray(L, rayPos, d, sum);
                }
            }
            direct = divs(sum, (float)K);
        }
        for (uint32_t i = 0; i < p->numDiffuse; i++) {
            if (doDiff) {
                L.sample = i;
                diff = add(diff, L.ambient);
                diffuse_ray(L, adds(tv.normal, EPS), rayPos, tv, p->time * (float)(i + 1u), diff);
                diff = add(diff, direct);
            }
        }
        if (doDiff) {
            const float den = indirect + (float)p->numDiffuse;
            diff.x = (tv.diff.x * indirect + diff.x) / den;
            diff.y = (tv.diff.y * indirect + diff.y) / den;
            diff.z = (tv.diff.z * indirect + diff.z) / den;
        }
    }
    outS = make_float4(gmin(gmax(spec.x, 0.0f), 1.0f), gmin(gmax(spec.y, 0.0f), 1.0f), gmin(gmax(spec.z, 0.0f), 1.0f), 0.0f);
    outD = make_float4(gmin(gmax(diff.x, 0.0f), 1.0f), gmin(gmax(diff.y, 0.0f), 1.0f), gmin(gmax(diff.z, 0.0f), 1.0f), 0.0f);
}

} // namespace dn
