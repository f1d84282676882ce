/*
 * dno_shapes.c -- TEST INFRASTRUCTURE (part of the CPU oracle, libdn_oracle.so): a restatement of the
 * reference's shape functions, src/DoonEngine/voxelShapes.c:23-442, used only to check the product's
 * GPU shape evaluation and host edits.  Not part of the product.
 *
 * The caller supplies each shape's transform and inverse (4x4, column-major); the oracle restates the
 * bounding box and chunk range (voxelShapes.c:93-177), the distance functions (23-89), the forward-
 * difference normal (131-147), the sphere's squared-distance test (239-333), and the edit rules
 * (191-231, 288-331) applied to a dense copy of the CPU map with the reference's DN_set_voxel /
 * DN_get_voxel / chunk-removal behaviour (voxel.c:1111-1161, 1289-1316).  Every float operation is
 * the reference's, in its order and type (fmin / fmax run in double where the reference calls them).
 */
#include "dn_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } sv3;

/* m * (x, y, z, w): ((c0 x + c1 y) + c2 z) + c3 w per component (quickmath.h:206-216) */
static sv3 sxf(const float m[4][4], float x, float y, float z, float w)
{
    sv3 r;
    r.x = m[0][0] * x + m[1][0] * y + m[2][0] * z + m[3][0] * w;
    r.y = m[0][1] * x + m[1][1] * y + m[2][1] * z + m[3][1] * w;
    r.z = m[0][2] * x + m[1][2] * y + m[2][2] * z + m[3][2] * w;
    return r;
}

static float l2(float x, float y) { return sqrtf(x * x + y * y); }
static float l3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }
static float qmax(float a, float b) { return a > b ? a : b; }   /* QM_MAX, quickmath.h:191 */

/* shape parameters derived once per shape */
typedef struct {
    int kind;
    float length[3], radius, radiusB, height, angles[2], radii[3];
} sdf_par;

static float sdf(const sdf_par* s, sv3 p)
{
    switch (s->kind) {
    case DNO_SHAPE_BOX:
    case DNO_SHAPE_ROUNDED_BOX: {   /* voxelShapes.c:23-37 */
        sv3 q = {(float)fabs(p.x) - s->length[0], (float)fabs(p.y) - s->length[1], (float)fabs(p.z) - s->length[2]};
        float q1 = l3(qmax(q.x, 0.0f), qmax(q.y, 0.0f), qmax(q.z, 0.0f));
        float q2 = (float)fmin(fmax(fmax(q.x, q.y), q.z), 0.0);
        float d = q1 + q2;
        return s->kind == DNO_SHAPE_BOX ? d : d - s->radius;
    }
    case DNO_SHAPE_TORUS:           /* 39-43 */
        return l2(l2(p.x, p.z) - s->radius, p.y) - s->radiusB;
    case DNO_SHAPE_ELLIPSOID:       /* 45-48 */
        return (float)((l3(p.x / s->radii[0], p.y / s->radii[1], p.z / s->radii[2]) - 1.0f) *
                       fmin(fmin(s->radii[0], s->radii[1]), s->radii[2]));
    case DNO_SHAPE_CYLINDER: {      /* 50-54 */
        float dx = l2(p.x, p.z) - s->radius, dy = (float)(fabs(p.y) - s->height);
        return (float)(fmin(fmax(dx, dy), 0.0) + l2(qmax(dx, 0.0f), qmax(dy, 0.0f)));
    }
    case DNO_SHAPE_CONE: {          /* 56-60 */
        float q = l2(p.x, p.z);
        return (float)fmax(s->angles[0] * q + s->angles[1] * p.y, -s->height - p.y);
    }
    case DNO_SHAPE_PYRAMID: {       /* 62-89 */
        float m2 = s->height * s->height * 0.25f;
        float px = fabsf(p.x) / s->length[0], pz = fabsf(p.z) / s->length[2], py = p.y;
        if (pz > px) { float t = px; px = pz; pz = t; }
        px -= 0.5f;
        pz -= 0.5f;
        sv3 q = {pz, s->height * py - 0.5f * px, s->height * px + 0.5f * py};
        float ss = fmaxf(-q.x, 0.0f);
        float t = fmaxf(fminf((q.y - 0.5f * pz) / (m2 + 0.25f), 0.0f), 1.0f);
        float a = m2 * (q.x + ss) * (q.x + ss) + q.y * q.y;
        float b = m2 * (q.x + 0.5f * t) * (q.x + 0.5f * t) + (q.y - m2 * t) * (q.y - m2 * t);
        float d2 = fminf(q.y, -q.x * m2 - q.y * 0.5f) > 0.0f ? 0.0f : fminf(a, b);
        return sqrtf((d2 + q.z * q.z) / m2) * (fmaxf(q.z, -py) >= 0.0f ? 1.0f : -1.0f);
    }
    }
    return 1.0f;
}

static sdf_par params_of(const dno_shape_op* op)
{
    sdf_par s;
    memset(&s, 0, sizeof(s));
    s.kind = op->kind;
    switch (op->kind) {
    case DNO_SHAPE_BOX: memcpy(s.length, op->v, 12); break;
    case DNO_SHAPE_ROUNDED_BOX: memcpy(s.length, op->v, 12); s.radius = op->a; break;
    case DNO_SHAPE_TORUS: s.radius = op->a; s.radiusB = op->b; break;
    case DNO_SHAPE_ELLIPSOID: memcpy(s.radii, op->v, 12); break;
    case DNO_SHAPE_CYLINDER: s.radius = op->a; s.height = op->b / 2; break;
    case DNO_SHAPE_CONE: {
        float hyp = sqrtf(op->a * op->a + op->b * op->b);
        s.angles[0] = op->b / hyp; s.angles[1] = op->a / hyp; s.height = op->b;
        break;
    }
    case DNO_SHAPE_PYRAMID: s.length[0] = op->v[0]; s.length[2] = op->v[2]; s.height = op->v[1]; break;
    }
    return s;
}

/* the local bounding box of each shape (voxelShapes.c:246-247, 341, 353-354, 368-369, 383-384,
 * 397-398, 420-421, 437-438) */
static void local_box(const dno_shape_op* op, sv3* mn, sv3* mx)
{
    const float* v = op->v;
    const float a = op->a, b = op->b;
    *mn = *mx = (sv3){0.0f, 0.0f, 0.0f};
    switch (op->kind) {
    case DNO_SHAPE_SPHERE: *mn = (sv3){op->c[0] - a, op->c[1] - a, op->c[2] - a}; *mx = (sv3){op->c[0] + a, op->c[1] + a, op->c[2] + a}; break;
    case DNO_SHAPE_BOX: *mn = (sv3){v[0] * -1.0f, v[1] * -1.0f, v[2] * -1.0f}; *mx = (sv3){v[0], v[1], v[2]}; break;
    case DNO_SHAPE_ROUNDED_BOX: *mn = (sv3){-v[0] - a, -v[1] - a, -v[2] - a}; *mx = (sv3){v[0] + a, v[0] + a, v[0] + a}; break;
    case DNO_SHAPE_TORUS: *mn = (sv3){-(a + b), -b, -(a + b)}; *mx = (sv3){a + b, b, a + b}; break;
    case DNO_SHAPE_ELLIPSOID: *mn = (sv3){-v[0], -v[1], -v[2]}; *mx = (sv3){v[0], v[1], v[2]}; break;
    case DNO_SHAPE_CYLINDER: *mn = (sv3){-a, -b / 2, -a}; *mx = (sv3){a, b / 2, a}; break;
    case DNO_SHAPE_CONE: *mn = (sv3){-a, -b, -a}; *mx = (sv3){a, 0.0f, a}; break;
    case DNO_SHAPE_PYRAMID: *mn = (sv3){-v[0] * 0.5f, 0.0f, -v[2] * 0.5f}; *mx = (sv3){v[0] * 0.5f, v[1], v[2] * 0.5f}; break;
    }
}

void dno_shape_bounds(const dno_shape_op* op, float mn[3], float mx[3])
{
    sv3 lo, hi;
    local_box(op, &lo, &hi);
    if (op->kind != DNO_SHAPE_SPHERE) {     /* voxelShapes.c:93-130 */
        const sv3 pts[8] = {{lo.x, lo.y, lo.z}, {lo.x, lo.y, hi.z}, {lo.x, hi.y, lo.z}, {lo.x, hi.y, hi.z},
                            {hi.x, lo.y, lo.z}, {hi.x, lo.y, hi.z}, {hi.x, hi.y, lo.z}, {hi.x, hi.y, hi.z}};
        float a[3] = {INFINITY, INFINITY, INFINITY}, b[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = 0; i < 8; i++) {
            sv3 t = sxf(op->transform, pts[i].x, pts[i].y, pts[i].z, 1.0f);
            const float c[3] = {t.x, t.y, t.z};
            for (int k = 0; k < 3; k++) {
                if (c[k] > b[k]) b[k] = c[k];
                if (c[k] < a[k]) a[k] = c[k];
            }
        }
        lo = (sv3){a[0], a[1], a[2]};
        hi = (sv3){b[0], b[1], b[2]};
    }
    mn[0] = lo.x; mn[1] = lo.y; mn[2] = lo.z;
    mx[0] = hi.x; mx[1] = hi.y; mx[2] = hi.z;
}

int dno_shape_range(const dno_shape_op* op, const uint32_t mapSize[3], int32_t cmin[3], int32_t cmax[3])
{
    /* voxelShapes.c:155-177: truncating division of the floor / ceil corners, clamped to the map */
    float mn[3], mx[3];
    dno_shape_bounds(op, mn, mx);
    const int grow = op->material == 255 ? 1 : 0;
    for (int k = 0; k < 3; k++) {
        int lo = (int)floorf(mn[k]) - grow, hi = (int)ceilf(mx[k]) + grow;
        int l = lo / 8, h = hi / 8;
        cmin[k] = l > 0 ? l : 0;
        cmax[k] = h < (int)mapSize[k] - 1 ? h : (int)mapSize[k] - 1;
        if (cmin[k] > cmax[k]) return 0;
    }
    return 1;
}

/* class of voxel (x, y, z): 0 untouched, 1 inside, 2 shell; normal before flipping */
static int classify(const dno_shape_op* op, const sdf_par* s, int x, int y, int z, float n[3])
{
    const int removing = op->material == 255;
    const float px = (float)x, py = (float)y, pz = (float)z;
    n[0] = n[1] = n[2] = 0.0f;
    if (op->kind == DNO_SHAPE_SPHERE) {
        const float r = op->a, r2 = r * r, r12 = (r + 1.0f) * (r + 1.0f);
        sv3 f = {px - op->c[0], py - op->c[1], pz - op->c[2]};
        float d2 = f.x * f.x + f.y * f.y + f.z * f.z;
        int cls = d2 < r2 ? 1 : (removing && op->flip && d2 < r12) ? 2 : 0;
        if (!cls || (cls == 1 && removing)) return cls;
        float m = (float)fmax(fmax(fabs(f.x), fabs(f.y)), fabs(f.z));
        float k = 1.0f / m;
        n[0] = f.x * k; n[1] = f.y * k; n[2] = f.z * k;
        return cls;
    }
    sv3 t = sxf(op->invTransform, px, py, pz, 1.0f);
    float dist = sdf(s, t);
    int cls = dist < 0.0f ? 1 : (dist < 1.0f && removing && op->flip) ? 2 : 0;
    if (!cls || (cls == 1 && removing)) return cls;
    const float h = 0.01f;
    float dx = sdf(s, sxf(op->invTransform, px + h, py + 0.0f, pz + 0.0f, 1.0f + 0.0f)) - dist;
    float dy = sdf(s, sxf(op->invTransform, px + 0.0f, py + h, pz + 0.0f, 1.0f + 0.0f)) - dist;
    float dz = sdf(s, sxf(op->invTransform, px + 0.0f, py + 0.0f, pz + h, 1.0f + 0.0f)) - dist;
    float m = (float)fmax(fmax(fabs(dx), fabs(dy)), fabs(dz));
    float k = 1.0f / m;
    n[0] = dx * k; n[1] = dy * k; n[2] = dz * k;
    return cls;
}

uint64_t dno_shape_eval(const dno_shape_op* op, const int32_t cmin[3], const int32_t cmax[3], uint32_t* counts,
                        dno_shape_hit* hits, uint64_t capacity)
{
    const sdf_par s = params_of(op);
    uint64_t total = 0;
    size_t chunk = 0;
    for (int mz = cmin[2]; mz <= cmax[2]; mz++)
    for (int my = cmin[1]; my <= cmax[1]; my++)
    for (int mx = cmin[0]; mx <= cmax[0]; mx++) {
        uint32_t n = 0;
        for (int z = 0; z < 8; z++)
        for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
            float nrm[3];
            int cls = classify(op, &s, mx * 8 + x, my * 8 + y, mz * 8 + z, nrm);
            if (!cls) continue;
            if (hits && total < capacity) {
                dno_shape_hit* e = &hits[total];
                e->local = (uint16_t)(x + 8 * (y + 8 * z));
                e->inside = cls == 1;
                e->pad = 0;
                memcpy(e->normal, nrm, 12);
            }
            total++;
            n++;
        }
        counts[chunk++] = n;
    }
    return total;
}

/* DN_compress_voxel (voxel.c:1289-1301): normal clamped with SSE min / max (a NaN component becomes 1) */
static uint32_t normal_word(uint8_t material, const float n[3])
{
    uint32_t b[3];
    for (int i = 0; i < 3; i++) {
        float v = n[i] < 1.0f ? n[i] : 1.0f;
        v = v > -1.0f ? v : -1.0f;
        b[i] = (uint32_t)(((int)(v * 255.0f) + 255) / 2);
    }
    return ((uint32_t)material << 24) | (b[0] << 16) | (b[1] << 8) | b[2];
}

/* DN_set_compressed_voxel on the dense map (voxel.c:1126-1161) */
static void dense_set(const uint32_t mapSize[3], uint32_t* nw, uint32_t* aw, int32_t* tileCount, int x, int y, int z,
                      uint32_t normal, uint32_t albedo)
{
    const uint32_t X = mapSize[0] * 8, Y = mapSize[1] * 8;
    const size_t t = (size_t)(x / 8) + mapSize[0] * ((size_t)(y / 8) + mapSize[1] * (size_t)(z / 8));
    const size_t v = (size_t)x + X * ((size_t)y + (size_t)Y * z);
    const int newEmpty = (normal >> 24) == 255;
    if (tileCount[t] == 0 && newEmpty) return;     /* no chunk and nothing to add */
    const int oldEmpty = (nw[v] >> 24) == 255;
    if (oldEmpty && !newEmpty) tileCount[t]++;
    else if (!oldEmpty && newEmpty) {
        if (--tileCount[t] <= 0) {                /* the chunk is removed: every voxel empty */
            tileCount[t] = 0;
            for (int cz = 0; cz < 8; cz++)
            for (int cy = 0; cy < 8; cy++)
            for (int cx = 0; cx < 8; cx++) {
                const size_t w = (size_t)((x / 8) * 8 + cx) + X * ((size_t)((y / 8) * 8 + cy) + (size_t)Y * ((z / 8) * 8 + cz));
                nw[w] = 0xFFFFFFFFu;
                aw[w] = 0;
            }
            return;
        }
    }
    nw[v] = normal;
    aw[v] = newEmpty ? 0u : albedo;
}

void dno_shape_apply(const dno_shape_op* op, const uint32_t mapSize[3], const int32_t cmin[3], const int32_t cmax[3],
                     const uint32_t* counts, const dno_shape_hit* hits, uint32_t* normalWords, uint32_t* albedoWords,
                     int32_t* tileCount)
{
    const int removing = op->material == 255;
    const uint32_t X = mapSize[0] * 8, Y = mapSize[1] * 8;
    const uint32_t albedo = ((uint32_t)op->albedo[0] << 24) | ((uint32_t)op->albedo[1] << 16) | ((uint32_t)op->albedo[2] << 8);
    size_t chunk = 0;
    uint64_t at = 0;
    for (int mz = cmin[2]; mz <= cmax[2]; mz++)
    for (int my = cmin[1]; my <= cmax[1]; my++)
    for (int mx = cmin[0]; mx <= cmax[0]; mx++) {
        const size_t t = (size_t)mx + mapSize[0] * ((size_t)my + mapSize[1] * (size_t)mz);
        const int tileExisted = tileCount[t] != 0;   /* the tile copied before the chunk's edits */
        const uint32_t n = counts[chunk++];
        for (uint32_t i = 0; i < n; i++) {
            const dno_shape_hit* e = &hits[at++];
            const int x = mx * 8 + (e->local & 7), y = my * 8 + ((e->local >> 3) & 7), z = mz * 8 + (e->local >> 6);
            const size_t v = (size_t)x + X * ((size_t)y + (size_t)Y * z);
            const int exists = tileCount[t] != 0 && (normalWords[v] >> 24) != 255;
            if (e->inside) {
                if (tileExisted && exists && !removing) continue;
                const uint32_t w = removing ? normal_word(op->material, op->normal) : normal_word(op->material, e->normal);
                dense_set(mapSize, normalWords, albedoWords, tileCount, x, y, z, w, albedo);
            } else {
                if (!tileExisted || !exists) continue;
                const float f[3] = {e->normal[0] * -1.0f, e->normal[1] * -1.0f, e->normal[2] * -1.0f};
                dense_set(mapSize, normalWords, albedoWords, tileCount, x, y, z,
                          normal_word((uint8_t)(normalWords[v] >> 24), f), albedoWords[v]);
            }
        }
    }
}
