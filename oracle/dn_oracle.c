/*
 * dn_oracle.c -- CPU oracle (test infrastructure; never linked by the product).
 *
 * Plain-C restatement of the reference's per-voxel lighting and draw path:
 *   voxelShared.comp   (DDA, voxel codec, rank/select, AABB, sky)
 *   voxelLighting.comp (specular / diffuse / shadow rays, running average)
 *   voxelDraw.comp     (primary rays, shading, view modes, gamma)
 *   voxel.c            (chunk packing 1391-1461, sync 719-786, requests 1463-1489,
 *                       stream state machine 1491-1536, voxel codec 1289-1316)
 * with the deterministic semantics D1..D15 listed in dn_oracle.h.  Every
 * floating-point expression keeps the reference's operation order; the file
 * must be compiled with -ffp-contract=off (no FMA contraction).
 */
#include "dn_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__FP_FAST_FMAF) && !defined(DNO_ALLOW_FMA)
/* contraction would change rounding; the build uses -ffp-contract=off */
#endif

#define EPS 0.0001f                  /* voxelShared.comp:7 */
#define INV_CHUNK 0.125f             /* voxelShared.comp:4 */
#define HALF_INV_CHUNK 0.0625f       /* voxelShared.comp:5 */
#define INV255 0.00392156862f        /* voxelShared.comp:249-253 */
#define MAT_EMPTY 255u

typedef struct { float x, y, z; } v3;
typedef struct { int32_t x, y, z; } iv3;

static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vmuls(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vadds(v3 a, float s) { return V(a.x + s, a.y + s, a.z + s); }
static inline v3 vdivv(v3 a, v3 b) { return V(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 vdivs(v3 a, float s) { return V(a.x / s, a.y / s, a.z / s); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* GLSL min/max: min(x,y) = y < x ? y : x ; max(x,y) = x < y ? y : x */
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }
static inline float gsign(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }
static inline v3 vnormalize(v3 v) { float l = sqrtf(dot3(v, v)); return vdivs(v, l); }
static inline v3 vabs(v3 v) { return V(fabsf(v.x), fabsf(v.y), fabsf(v.z)); }
static inline v3 vfloor(v3 v) { return V(floorf(v.x), floorf(v.y), floorf(v.z)); }
static inline float min3(v3 v) { return gmin(gmin(v.x, v.y), v.z); }
/* reflect(I, N) = I - 2*dot(N, I)*N */
static inline v3 vreflect(v3 I, v3 N) { float t = 2.0f * dot3(N, I); return vsub(I, vmuls(N, t)); }
/* refract(I, N, eta) per the GLSL specification */
static inline v3 vrefract(v3 I, v3 N, float eta)
{
    float d = dot3(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return V(0.0f, 0.0f, 0.0f);
    float s = eta * d + sqrtf(k);
    return vsub(vmuls(I, eta), vmuls(N, s));
}
/* float -> int32 with saturation and NaN -> 0 */
static inline int32_t f2i(float x)
{
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT_MAX;
    if (x < -2147483648.0f) return INT_MIN;
    return (int32_t)x;
}

/* ---------------------------------------------------------------- RNG (D5) */

uint32_t dno_hash32(uint32_t x)
{
    /* 32-bit integer finaliser ("lowbias32", C. Wellons' hash-prospector) */
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

static inline uint32_t rng_key(uint32_t seed, uint32_t mapId, uint32_t voxel)
{
    return dno_hash32(seed ^ dno_hash32(voxel ^ dno_hash32(mapId + 0x632be5abu)));
}

static inline float hrand(uint32_t key, uint32_t stream, uint32_t idx)
{
    uint32_t h = dno_hash32(key ^ dno_hash32((stream << 28) ^ idx));
    return (float)(h >> 8) * (1.0f / 8388608.0f) - 1.0f;   /* exact, in [-1, 1) */
}

/* deterministic sine: Cody-Waite reduction by pi/2 (three-part constant) and
 * Taylor polynomials on [-pi/4, pi/4]. */
float dno_sin(float x)
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
    switch (q) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
    }
}

static inline float fractf(float x) { return x - floorf(x); }
/* rand(seed) = fract(sin(seed) * 43758.5453) * 2 - 1 (voxelLighting.comp:29-32) */
static inline float srand1(float s) { return fractf(dno_sin(s) * 43758.5453f) * 2.0f - 1.0f; }

/* rand_unit_sphere, mode A (voxelLighting.comp:47-57; D6 bound) */
static v3 sphere_sin(float seed)
{
    for (int t = 0; t < 64; t++) {
        float s = seed;
        seed = seed + 1.0f;
        v3 p = V(srand1(s), srand1(s * 2.0f), srand1(s * 3.0f));
        if (dot3(p, p) >= 1.0f) continue;
        return p;
    }
    return V(0.0f, 0.0f, 0.0f);
}

/* rand_unit_sphere, mode B */
static v3 sphere_hash(uint32_t key, uint32_t stream, uint32_t base)
{
    for (uint32_t t = 0; t < 64; t++) {
        uint32_t i = (base << 8) | (3u * t);
        v3 p = V(hrand(key, stream, i), hrand(key, stream, i + 1u), hrand(key, stream, i + 2u));
        if (dot3(p, p) >= 1.0f) continue;
        return p;
    }
    return V(0.0f, 0.0f, 0.0f);
}

void dno_sphere_points(uint32_t K, float out[][3])
{
    /* golden-angle Fibonacci sphere: y_k = 1 - 2k/(K-1), theta_k = k*pi*(3-sqrt(5)) */
    const double ga = 3.14159265358979323846 * (3.0 - sqrt(5.0));
    for (uint32_t k = 0; k < K; k++) {
        double y = (K > 1) ? 1.0 - 2.0 * (double)k / (double)(K - 1) : 1.0;
        double r = sqrt(fmax(0.0, 1.0 - y * y));
        double th = ga * (double)k;
        out[k][0] = (float)(cos(th) * r);
        out[k][1] = (float)y;
        out[k][2] = (float)(sin(th) * r);
    }
}

/* ------------------------------------------------------------ voxel codec */

void dno_compress_voxel(uint8_t material, const float normal[3], const uint8_t albedo[3], dno_cvoxel* out)
{
    /* voxel.c:1289-1301: clamp to [-1,1], byte = ((int)(n*255)+255)/2 */
    uint32_t nb[3];
    for (int i = 0; i < 3; i++) {
        float n = normal[i];
        n = (n < 1.0f) ? n : 1.0f;
        n = (n > -1.0f) ? n : -1.0f;
        nb[i] = (uint32_t)(((int)(n * 255.0f) + 255) / 2);
    }
    out->normal = ((uint32_t)material << 24) | (nb[0] << 16) | (nb[1] << 8) | nb[2];
    out->albedo = ((uint32_t)albedo[0] << 24) | ((uint32_t)albedo[1] << 16) | ((uint32_t)albedo[2] << 8);
}

void dno_decompress_voxel(dno_cvoxel v, uint8_t* material, float normal[3], uint8_t albedo[3])
{
    /* voxel.c:1303-1316 */
    const float inv255 = 1.0f / 255.0f;
    int32_t n[3] = {(int32_t)((v.normal >> 16) & 0xFF), (int32_t)((v.normal >> 8) & 0xFF), (int32_t)(v.normal & 0xFF)};
    for (int i = 0; i < 3; i++) normal[i] = (float)(n[i] * 2 - 255) * inv255;
    *material = (uint8_t)(v.normal >> 24);
    albedo[0] = (uint8_t)((v.albedo >> 24) & 0xFF);
    albedo[1] = (uint8_t)((v.albedo >> 16) & 0xFF);
    albedo[2] = (uint8_t)((v.albedo >> 8) & 0xFF);
}

/* ---------------------------------------------------------- chunk packing */

static int face_visible(const dno_chunk* c, const dno_material* mats, int x, int y, int z)
{
    /* _DN_check_face_visible, voxel.c:1391-1394 */
    if (x < 0 || y < 0 || z < 0 || x >= 8 || y >= 8 || z >= 8) return 1;
    uint32_t m = c->voxels[x][y][z].normal >> 24;
    return m == MAT_EMPTY || mats[m].opacity < 1.0f;
}

void dno_pack_chunk(const dno_chunk* c, const dno_material* mats, dno_packed* out)
{
    /* _DN_chunk_to_gpu, voxel.c:1397-1461 */
    memset(out->mask, 0, sizeof(out->mask));
    memset(out->partial, 0, sizeof(out->partial));
    uint32_t n = 0;
    for (int z = 0; z < 8; z++)
    for (int y = 0; y < 8; y++)
    for (int x = 0; x < 8; x++) {
        uint32_t index = (uint32_t)(x + 8 * (y + 8 * z));
        if ((index & 31) == 0 && index != 0 && ((index >> 5) & 3) == 0)
            out->partial[(index >> 7) - 1] = n;
        uint32_t nw = c->voxels[x][y][z].normal;
        if ((nw >> 24) == MAT_EMPTY) continue;
        int vis = face_visible(c, mats, x + 1, y, z) || face_visible(c, mats, x - 1, y, z) ||
                  face_visible(c, mats, x, y + 1, z) || face_visible(c, mats, x, y - 1, z) ||
                  face_visible(c, mats, x, y, z + 1) || face_visible(c, mats, x, y, z - 1);
        if (!vis) continue;
        out->mask[index >> 5] |= 1u << (index & 31);
        uint32_t a = c->voxels[x][y][z].albedo;
        float lr = (float)((a >> 24) & 0xFF) * 0.00392156862f;
        float lg = (float)((a >> 16) & 0xFF) * 0.00392156862f;
        float lb = (float)((a >> 8) & 0xFF) * 0.00392156862f;
        lr = powf(lr, 2.2f); lg = powf(lg, 2.2f); lb = powf(lb, 2.2f);
        lr = lr * 255.0f; lg = lg * 255.0f; lb = lb * 255.0f;
        uint32_t r = (uint8_t)lr, g = (uint8_t)lg, b = (uint8_t)lb;
        out->vox[n][0] = nw;
        out->vox[n][1] = (r << 24) | (g << 16) | (b << 8);
        n++;
    }
    out->nvox = n;
}

/* ---------------------------------------------------------------- map state */

typedef struct orec {
    uint32_t mask[16];
    uint32_t partial[3];
    uint32_t nvox;
    uint32_t samples;
    uint32_t (*vox)[2];
    float (*diff)[3];
    float (*spec)[3];
} orec;

/* a node of the reference's GPU voxel buffer (DNvoxelNode, voxel.h:74-79); tile -1 = unused */
typedef struct onode { uint32_t size; uint64_t start; int64_t tile; } onode;

struct dno_map {
    uint32_t sx, sy, sz;
    uint64_t ntiles;
    uint8_t* state;     /* 0 absent, 1 unloaded, 2 loaded, 3 requested */
    uint8_t* vis;
    uint8_t* touch;
    uint32_t* lastUsed;
    orec* rec;
    uint32_t frameNum;
    uint32_t* req;
    uint32_t nreq, reqCap;
    dno_counters ctr;
    /* LRU residency (the reference's node buffer) */
    int lru;
    onode* nodes;
    size_t nnodes, nodesCap;
    uint64_t voxelCap, chunkCap;
};

static void rec_free(orec* r)
{
    free(r->vox); free(r->diff); free(r->spec);
    memset(r, 0, sizeof(*r));
}

dno_map* dno_create(uint32_t sx, uint32_t sy, uint32_t sz)
{
    dno_map* m = (dno_map*)calloc(1, sizeof(dno_map));
    if (!m) return NULL;
    m->sx = sx; m->sy = sy; m->sz = sz;
    m->ntiles = (uint64_t)sx * sy * sz;
    m->state = (uint8_t*)calloc(m->ntiles, 1);
    m->vis = (uint8_t*)calloc(m->ntiles, 1);
    m->touch = (uint8_t*)calloc(m->ntiles, 1);
    m->lastUsed = (uint32_t*)calloc(m->ntiles, 4);
    m->rec = (orec*)calloc(m->ntiles, sizeof(orec));
    if (!m->state || !m->vis || !m->touch || !m->lastUsed || !m->rec) { dno_destroy(m); return NULL; }
    return m;
}

void dno_destroy(dno_map* m)
{
    if (!m) return;
    if (m->rec) for (uint64_t t = 0; t < m->ntiles; t++) rec_free(&m->rec[t]);
    free(m->state); free(m->vis); free(m->touch); free(m->lastUsed); free(m->rec); free(m->req);
    free(m->nodes);
    free(m);
}

static void rec_load(orec* r, const dno_chunk* c, const dno_material* mats)
{
    dno_packed* p = (dno_packed*)malloc(sizeof(dno_packed));
    dno_pack_chunk(c, mats, p);
    rec_free(r);
    memcpy(r->mask, p->mask, sizeof(r->mask));
    memcpy(r->partial, p->partial, sizeof(r->partial));
    r->nvox = p->nvox;
    r->samples = 0;
    uint32_t n = p->nvox ? p->nvox : 1;
    r->vox = malloc(sizeof(uint32_t[2]) * n);
    r->diff = calloc(n, sizeof(float[3]));
    r->spec = calloc(n, sizeof(float[3]));
    memcpy(r->vox, p->vox, sizeof(uint32_t[2]) * p->nvox);
    free(p);
}

static void push_req(dno_map* m, uint32_t w)
{
    if (m->nreq == m->reqCap) {
        m->reqCap = m->reqCap ? m->reqCap * 2 : 1024;
        m->req = (uint32_t*)realloc(m->req, sizeof(uint32_t) * m->reqCap);
    }
    m->req[m->nreq++] = w;
}

/* ---------------------------------------------- LRU residency (node buffer) */

static void nodes_reserve(dno_map* m, size_t n)
{
    if (n <= m->nodesCap) return;
    size_t c = m->nodesCap ? m->nodesCap : 64;
    while (c < n) c *= 2;
    m->nodes = (onode*)realloc(m->nodes, c * sizeof(onode));
    m->nodesCap = c;
}

/* DN_set_max_voxels_gpu's node part (voxel.c:1064-1079): (num - voxelCap) / 512 whole nodes appended */
static void nodes_grow(dno_map* m, uint64_t num)
{
    if (num <= m->voxelCap) return;
    int numNewNodes = (int)((num - m->voxelCap) / 512);
    nodes_reserve(m, m->nnodes + (size_t)numNewNodes);
    for (int i = 0; i < numNewNodes; i++) {
        onode* nd = &m->nodes[m->nnodes + (size_t)i];
        nd->tile = -1;
        nd->size = 512;
        nd->start = m->voxelCap + (uint64_t)i * 512;
    }
    m->nnodes += (size_t)numNewNodes;
    m->voxelCap = num;
}

void dno_set_lru(dno_map* m, uint64_t numChunks)
{
    /* DN_create_volume's buffer (voxel.c:181, 190, 235-249): 512 * numChunks / 2 voxels of 512-voxel nodes */
    m->lru = 1;
    m->voxelCap = 512 * numChunks / 2;
    m->nnodes = (size_t)(m->voxelCap / 512);
    nodes_reserve(m, m->nnodes ? m->nnodes : 1);
    for (size_t i = 0; i < m->nnodes; i++) {
        m->nodes[i].tile = -1;
        m->nodes[i].size = 512;
        m->nodes[i].start = (uint64_t)i * 512;
    }
    m->chunkCap = numChunks;
}

void dno_set_chunk_cap(dno_map* m, uint64_t chunkCap) { m->chunkCap = chunkCap; }

size_t dno_lru_nodes(const dno_map* m, uint64_t* voxelCap, uint32_t* sizes, uint64_t* starts, int64_t* tiles, size_t cap)
{
    if (voxelCap) *voxelCap = m->lru ? m->voxelCap : 0;
    if (!m->lru) return 0;
    for (size_t i = 0; i < m->nnodes && i < cap; i++) {
        if (sizes) sizes[i] = m->nodes[i].size;
        if (starts) starts[i] = m->nodes[i].start;
        if (tiles) tiles[i] = m->nodes[i].tile;
    }
    return m->nnodes;
}

/* _DN_unload_voxels (voxel.c:1538-1546) */
static void lru_unload(dno_map* m, int64_t tile)
{
    for (size_t i = 0; i < m->nnodes; i++)
        if (m->nodes[i].tile == tile) { m->nodes[i].tile = -1; break; }
}

/* _DN_stream_voxels (voxel.c:1554-1640) without the upload: 1 with a node (*victim = the tile whose node was
 * taken, or -1), 0 without (the buffer must grow).  The reference compares the unsigned node size with its
 * int best size, which starts at -1: as unsigned that is the largest value. */
static int lru_stream(dno_map* m, int64_t tile, uint32_t numVoxels, int64_t* victim)
{
    *victim = -1;
    int nodeSize = 16;
    while (nodeSize < (int)numVoxels) nodeSize *= 2;
    uint32_t maxTime = 0;
    int maxTimeNodeSize = -1;
    long maxTimeIndex = -1;
    for (size_t i = 0; i < m->nnodes; i++) {
        if (m->nodes[i].size < (uint32_t)nodeSize) continue;
        uint32_t time = m->nodes[i].tile >= 0 ? m->lastUsed[m->nodes[i].tile] : UINT32_MAX;
        if (time > maxTime || (time == UINT32_MAX && m->nodes[i].size < (uint32_t)maxTimeNodeSize)) {
            maxTime = time;
            maxTimeNodeSize = (int)m->nodes[i].size;
            maxTimeIndex = (long)i;
        }
        if (maxTimeNodeSize == nodeSize && maxTime == UINT32_MAX) break;
    }
    if (maxTimeIndex < 0 || maxTime <= 1) return 0;
    *victim = m->nodes[maxTimeIndex].tile;
    if (maxTimeNodeSize > nodeSize) {
        int numAdded = 0;
        while (maxTimeNodeSize > nodeSize) { maxTimeNodeSize /= 2; numAdded++; }
        nodes_reserve(m, m->nnodes + (size_t)numAdded);
        uint64_t orgStart = m->nodes[maxTimeIndex].start;
        memmove(&m->nodes[maxTimeIndex + numAdded], &m->nodes[maxTimeIndex], sizeof(onode) * (m->nnodes - (size_t)maxTimeIndex));
        uint32_t mult = 1;
        for (long i = maxTimeIndex; i <= maxTimeIndex + numAdded; i++) {
            m->nodes[i].size = (uint32_t)nodeSize * mult;
            m->nodes[i].start = orgStart + (i == maxTimeIndex ? 0 : (uint64_t)nodeSize * mult);
            m->nodes[i].tile = -1;
            if (i > maxTimeIndex) mult *= 2;
        }
        m->nnodes += (size_t)numAdded;
    }
    m->nodes[maxTimeIndex].tile = tile;
    return 1;
}

/* _DN_sort_gpu_voxel_buffer (voxel.c:1642-1695); with no node the loop does not run (the reference's
 * size_t count minus one would wrap) */
static void lru_sort(dno_map* m, int maxCopies)
{
    int numCopies = 0;
    for (size_t i = 0; m->nnodes > 0 && i < m->nnodes - 1; i++) {
        onode cur = m->nodes[i], next = m->nodes[i + 1];
        if (cur.tile >= 0) continue;
        if (next.tile >= 0 || next.size < cur.size) {
            numCopies++;
            next.start -= cur.size;
            cur.start += next.size;
            m->nodes[i] = next;
            m->nodes[i + 1] = cur;
        }
        if (next.tile < 0 && cur.size == next.size && cur.size < 512) {
            numCopies++;
            m->nodes[i].size *= 2;
            if (i < m->nnodes - 2) memmove(&m->nodes[i + 1], &m->nodes[i + 2], sizeof(onode) * (m->nnodes - i - 2));
            m->nnodes--;
        }
        if (numCopies > maxCopies) break;
    }
}

/* the node model's steps on their own, for a differential test against the product's model */
int dno_lru_stream(dno_map* m, int64_t tile, uint32_t nvox, int64_t* victim) { return lru_stream(m, tile, nvox, victim); }
void dno_lru_unload(dno_map* m, int64_t tile) { lru_unload(m, tile); }
void dno_lru_sort(dno_map* m, int maxCopies) { lru_sort(m, maxCopies); }
void dno_lru_grow(dno_map* m, uint64_t num) { nodes_grow(m, num); }
void dno_set_last_used(dno_map* m, const uint32_t* lastUsed) { memcpy(m->lastUsed, lastUsed, m->ntiles * sizeof(uint32_t)); }

void dno_sync(dno_map* m, const dno_handle* cpuMap, const dno_chunk* chunks,
              const dno_material* mats, int op, int split)
{
    /* DN_sync_gpu, voxel.c:719-786 */
    if (split < 1) split = 1;
    m->frameNum++;
    if (m->frameNum >= (uint32_t)split) m->frameNum = 0;
    m->nreq = 0;
    int resizeVoxels = 0;
    /* lastUsed: rays set it to 0 during the frame (D4: when entering a loaded chunk), so every tile's value
     * is 0 before the loop reaches it; the loop adds 1 */
    for (uint64_t t = 0; t < m->ntiles; t++) {
        if (m->touch[t]) m->lastUsed[t] = 0;
        m->touch[t] = 0;
    }
    for (uint64_t t = 0; t < m->ntiles; t++) {
        int gflag = m->state[t];
        int vis = m->vis[t];
        if (m->lastUsed[t] != 0xFFFFFFFFu) m->lastUsed[t]++;
        int exists = cpuMap[t].flag != 0;
        int updated = exists ? chunks[cpuMap[t].chunkIndex].updated != 0 : 0;
        /* _DN_request_chunk_lighting, voxel.c:1463-1489 (D4: visible cleared here) */
        if (op != 1 && gflag == 2 && vis && (((uint32_t)(t % (uint64_t)split) == m->frameNum) || updated)) {
            for (uint32_t i = 0; i < m->rec[t].nvox; i += 32) push_req(m, ((uint32_t)t << 4) | (i / 32));
            vis = 0;
        }
        /* _DN_stream_to_gpu, voxel.c:1491-1536 */
        if (op != 0) {
            /* every assignment of the reference's flags word clears the visible bit */
            int changed = 0;
            if (exists && gflag == 0) { gflag = 1; changed = 1; }
            else if (!exists && gflag != 0) {
                if (gflag == 2) { rec_free(&m->rec[t]); if (m->lru) lru_unload(m, (int64_t)t); }
                gflag = 0; changed = 1;
            }
            if (gflag == 2 && updated) { rec_free(&m->rec[t]); if (m->lru) lru_unload(m, (int64_t)t); gflag = 3; changed = 1; }
            if (gflag == 3 && exists) {
                rec_load(&m->rec[t], &chunks[cpuMap[t].chunkIndex], mats);
                gflag = 2; m->lastUsed[t] = 0; changed = 1;
                if (m->lru) {
                    int64_t victim;
                    if (!lru_stream(m, (int64_t)t, m->rec[t].nvox, &victim)) {
                        /* no node: the chunk stays unloaded and the buffer grows after the loop */
                        rec_free(&m->rec[t]);
                        gflag = 1;
                        resizeVoxels = 1;
                    } else if (victim >= 0) {
                        /* the node's chunk is unloaded (its flags word set to 1, which clears the visible
                         * bit); its voxels are gone and a later load packs it again */
                        m->state[victim] = 1;
                        m->vis[victim] = 0;
                        rec_free(&m->rec[victim]);
                    }
                }
            }
            if (changed) vis = 0;
        }
        m->state[t] = (uint8_t)gflag;
        m->vis[t] = (uint8_t)vis;
    }
    if (m->lru) {
        lru_sort(m, 10);
        if (resizeVoxels) {
            uint64_t newCap = m->voxelCap * 2 < m->chunkCap * 512 ? m->voxelCap * 2 : m->chunkCap * 512;
            nodes_grow(m, newCap);
        }
    }
}

/* ------------------------------------------------------------------- DDA */

typedef struct voxel {
    v3 normal; uint32_t material; v3 albedo; v3 spec; v3 diff;
} voxel;

typedef struct tstate { uint32_t lastVoxID; float lastVoxRefract; } tstate;

typedef struct ctx {
    const dno_map* m;
    const dno_material* mats;
    v3 sunStrength;
    float emissive;   /* D9 */
    int refraction;
    v3 orgRayPos;
    dno_counters c;
    uint32_t segSteps;  /* cells visited by the current step_map call (D16) */
    int capped;
} ctx;

/* D16: a segment whose direction has a zero or NaN component (its reciprocal is then infinite or NaN)
 * traverses nothing: it ends at once as a miss.  In the reference such a ray makes a side distance NaN
 * (0 * inf) after one step, after which no axis can step and its loops (voxelShared.comp:339, 435) never
 * end; reflect() without an added EPSILON (voxelLighting.comp:132, 163) produces them.  A segment that
 * has visited step_cap cells also ends as a miss: with a finite direction that bound is never reached
 * without refraction (at most sx+sy+sz chunk cells, 24 voxel cells per chunk entered); it ends repeated
 * refraction inside transparent voxels. */
static inline int finite_dir(v3 inv) { return isfinite(inv.x) && isfinite(inv.y) && isfinite(inv.z); }
static inline uint32_t step_cap(uint32_t sx, uint32_t sy, uint32_t sz)
{
    uint64_t c = 256ull * ((uint64_t)sx + sy + sz) + 4096ull;
    return c > (1ull << 23) ? (1u << 23) : (uint32_t)c;
}

/* idempotent flag store: written only when it changes, so that threads whose rays cross the same tiles do not
 * keep invalidating each other's cache lines with stores of the value already there */
static inline void store_u8(uint8_t* p, uint8_t v)
{
    if (__atomic_load_n(p, __ATOMIC_RELAXED) != v) __atomic_store_n(p, v, __ATOMIC_RELAXED);
}
static inline uint8_t load_u8(const uint8_t* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }

static inline uint32_t map_index(const dno_map* m, iv3 p)
{
    return (uint32_t)p.x + m->sx * ((uint32_t)p.y + m->sy * (uint32_t)p.z);
}
static inline int in_map(const dno_map* m, iv3 p)
{
    return p.x >= 0 && p.y >= 0 && p.z >= 0 && (uint32_t)p.x < m->sx && (uint32_t)p.y < m->sy && (uint32_t)p.z < m->sz;
}
static inline int in_chunk(iv3 p) { return p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < 8 && p.y < 8 && p.z < 8; }

static inline int vox_exists(const orec* r, iv3 p)
{
    uint32_t i = (uint32_t)(p.x + 8 * (p.y + 8 * p.z));
    return (r->mask[i >> 5] >> (i & 31)) & 1u;
}
/* rank of a set bit (get_voxel_index, voxelShared.comp:150-169) */
static inline uint32_t vox_rank(const orec* r, iv3 p)
{
    uint32_t li = (uint32_t)(p.x + 8 * (p.y + 8 * p.z));
    uint32_t w = li >> 5;
    uint32_t n = (w > 3) ? r->partial[(w >> 2) - 1] : 0;
    for (uint32_t i = w & ~3u; i <= w; i++) {
        uint32_t bits = r->mask[i];
        if (i == w) bits &= (1u << (li & 31)) - 1u;
        n += (uint32_t)__builtin_popcount(bits);
    }
    return n;
}
/* select (get_voxel_position, voxelShared.comp:172-224): position of the n-th set bit */
static inline int vox_select(const orec* r, uint32_t n, iv3* out)
{
    uint32_t count = 0;
    for (uint32_t w = 0; w < 16; w++) {
        uint32_t bits = r->mask[w];
        uint32_t c = (uint32_t)__builtin_popcount(bits);
        if (count + c > n) {
            for (uint32_t b = 0; b < 32; b++) {
                if ((bits >> b) & 1u) {
                    if (count == n) {
                        uint32_t pos = w * 32 + b;
                        out->x = (int32_t)(pos % 8); out->y = (int32_t)((pos / 8) % 8); out->z = (int32_t)(pos / 64);
                        return 1;
                    }
                    count++;
                }
            }
        }
        count += c;
    }
    out->x = out->y = out->z = -1;
    return 0;
}

static inline void decompress(const orec* r, uint32_t rank, voxel* v)
{
    /* decompress_voxel, voxelShared.comp:236-256 (FP32 lighting, D3) */
    uint32_t nw = r->vox[rank][0], aw = r->vox[rank][1];
    v->normal = V(((float)((nw >> 16) & 0xFF) * INV255 - 0.5f) * 2.0f,
                  ((float)((nw >> 8) & 0xFF) * INV255 - 0.5f) * 2.0f,
                  ((float)(nw & 0xFF) * INV255 - 0.5f) * 2.0f);
    v->material = nw >> 24;
    v->albedo = V((float)((aw >> 24) & 0xFF) * INV255, (float)((aw >> 16) & 0xFF) * INV255,
                  (float)((aw >> 8) & 0xFF) * INV255);
    v->diff = V(r->diff[rank][0], r->diff[rank][1], r->diff[rank][2]);
    v->spec = V(r->spec[rank][0], r->spec[rank][1], r->spec[rank][2]);
}

/* init_DDA, voxelShared.comp:300-306 */
static inline void init_dda(v3 dir, v3 inv, v3 p, iv3* pos, v3* delta, iv3* step, v3* side)
{
    v3 fl = vfloor(p);
    pos->x = f2i(fl.x); pos->y = f2i(fl.y); pos->z = f2i(fl.z);
    *delta = vabs(inv);
    v3 s = V(gsign(dir.x), gsign(dir.y), gsign(dir.z));
    step->x = f2i(s.x); step->y = f2i(s.y); step->z = f2i(s.z);
    side->x = (s.x * ((float)pos->x - p.x) + s.x * 0.5f + 0.5f) * delta->x;
    side->y = (s.y * ((float)pos->y - p.y) + s.y * 0.5f + 0.5f) * delta->y;
    side->z = (s.z * ((float)pos->z - p.z) + s.z * 0.5f + 0.5f) * delta->z;
}

/* iterate_DDA, voxelShared.comp:309-317 */
static inline void iter_dda(v3 delta, iv3 step, v3* side, iv3* pos, v3* normal)
{
    int mx = side->x <= gmin(side->y, side->z);
    int my = side->y <= gmin(side->z, side->x);
    int mz = side->z <= gmin(side->x, side->y);
    float fx = mx ? 1.0f : 0.0f, fy = my ? 1.0f : 0.0f, fz = mz ? 1.0f : 0.0f;
    side->x = side->x + fx * delta.x;
    side->y = side->y + fy * delta.y;
    side->z = side->z + fz * delta.z;
    pos->x += mx * step.x; pos->y += my * step.y; pos->z += mz * step.z;
    normal->x = fx * (float)(-step.x);
    normal->y = fy * (float)(-step.y);
    normal->z = fz * (float)(-step.z);
}

typedef struct hitinfo { uint32_t tile; iv3 local; } hitinfo;

/* step_chunk, voxelShared.comp:328-418 */
static int step_chunk(ctx* c, tstate* ts, iv3 mapPos, uint32_t tile, v3* rayDir, v3* inv, v3* rayPos,
                      int ignoreFirst, float maxDepth, v3* hitNormal, voxel* vox,
                      v3* colorAdd, float* colorMult, int* refracted, hitinfo* hi)
{
    const orec* r = &c->m->rec[tile];
    *refracted = 0;
    iv3 pos, step; v3 delta, side, lastSide = V(0.0f, 0.0f, 0.0f);
    init_dda(*rayDir, *inv, *rayPos, &pos, &delta, &step, &side);
    const uint32_t cap = step_cap(c->m->sx, c->m->sy, c->m->sz);
    while (in_chunk(pos)) {
        if (c->segSteps >= cap) { c->capped = 1; return 0; }
        c->segSteps++;
        c->c.innerSteps++;
        if (vox_exists(r, pos) && !ignoreFirst) {
            uint32_t rank = vox_rank(r, pos);
            c->c.hits++;
            decompress(r, rank, vox);
            const dno_material* mat = &c->mats[vox->material];
            uint32_t thisID = (r->vox[rank][1] & 0xFFFFFF00u) | (r->vox[rank][0] >> 24);
            if (mat->opacity == 1.0f) {
                float t = min3(lastSide) + EPS;
                *rayPos = vadd(*rayPos, vmuls(*rayDir, t));
                hi->tile = tile; hi->local = pos;
                return 1;
            } else if (ts->lastVoxID != thisID) {
                v3 cur = vadd(*rayPos, vmuls(*rayDir, min3(lastSide)));
                cur = vadd(V((float)mapPos.x, (float)mapPos.y, (float)mapPos.z), vmuls(cur, INV_CHUNK));
                v3 to = vsub(cur, c->orgRayPos);
                if (maxDepth < 0.0f || dot3(to, to) < maxDepth * maxDepth) {
                    float k = *colorMult * mat->opacity;
                    colorAdd->x = colorAdd->x + k * vox->albedo.x * c->sunStrength.x;
                    colorAdd->y = colorAdd->y + k * vox->albedo.y * c->sunStrength.y;
                    colorAdd->z = colorAdd->z + k * vox->albedo.z * c->sunStrength.z;
                    *colorMult = *colorMult * (1.0f - mat->opacity);
                }
                float rd = min3(lastSide);
                if (c->refraction && rd > 0.0f) {
                    *refracted = 1;
                    *rayPos = vadd(*rayPos, vmuls(*rayDir, rd + EPS));
                    v3 n = (dot3(vox->normal, *rayDir) < 0.0f) ? vnormalize(vox->normal) : *hitNormal;
                    *rayDir = vrefract(*rayDir, n, ts->lastVoxRefract / mat->refractIndex);
                    *inv = V(1.0f / rayDir->x, 1.0f / rayDir->y, 1.0f / rayDir->z);
                    if (!finite_dir(*inv)) { c->c.degenerate++; c->capped = 1; return 0; }
                    init_dda(*rayDir, *inv, *rayPos, &pos, &delta, &step, &side);
                    lastSide = V(0.0f, 0.0f, 0.0f);
                }
                ts->lastVoxID = thisID;
                ts->lastVoxRefract = mat->refractIndex;
            }
        } else if (ts->lastVoxID != 255u) {
            if (c->refraction) {
                *refracted = 1;
                *rayPos = vadd(*rayPos, vmuls(*rayDir, min3(lastSide) + EPS));
                v3 old = *rayDir;
                v3 nn = V(-vox->normal.x, -vox->normal.y, -vox->normal.z);
                v3 n = (dot3(nn, *rayDir) < 0.0f) ? vnormalize(nn) : *hitNormal;
                *rayDir = vrefract(*rayDir, n, ts->lastVoxRefract);
                if (rayDir->x == 0.0f && rayDir->y == 0.0f && rayDir->z == 0.0f) *rayDir = old;
                *inv = V(1.0f / rayDir->x, 1.0f / rayDir->y, 1.0f / rayDir->z);
                if (!finite_dir(*inv)) { c->c.degenerate++; c->capped = 1; return 0; }
                init_dda(*rayDir, *inv, *rayPos, &pos, &delta, &step, &side);
                lastSide = V(0.0f, 0.0f, 0.0f);
            }
            ts->lastVoxID = 255u;
            ts->lastVoxRefract = 1.0f;
        }
        lastSide = side;
        iter_dda(delta, step, &side, &pos, hitNormal);
        ignoreFirst = 0;
    }
    return 0;
}

/* step_map, voxelShared.comp:421-475 */
static int step_map(ctx* c, tstate* ts, v3* rayDir, v3 inv, v3* rayPos, int ignoreFirst, float maxDepth,
                    v3* hitNormal, voxel* vox, v3* colorAdd, float* colorMult, hitinfo* hi)
{
    const dno_map* m = c->m;
    int requested = 0;
    *colorAdd = V(0.0f, 0.0f, 0.0f);
    *colorMult = 1.0f;
    c->c.rays++;
    c->segSteps = 0;
    c->capped = 0;
    if (!finite_dir(inv)) { c->c.degenerate++; return 0; }
    const uint32_t cap = step_cap(m->sx, m->sy, m->sz);
    iv3 pos, step; v3 delta, side, lastSide = V(0.0f, 0.0f, 0.0f);
    init_dda(*rayDir, inv, *rayPos, &pos, &delta, &step, &side);
    while (in_map(m, pos)) {
        if (c->segSteps >= cap) return 0;
        c->segSteps++;
        c->c.outerSteps++;
        uint32_t t = map_index(m, pos);
        uint8_t st = load_u8(&m->state[t]);
        if (st == 2) {
            c->c.chunksEntered++;
            store_u8(&m->touch[t], 1);
            float tt = min3(lastSide) - EPS;
            v3 up = vadd(*rayPos, vmuls(*rayDir, tt));
            v3 cp = V((up.x - (float)pos.x) * 8.0f, (up.y - (float)pos.y) * 8.0f, (up.z - (float)pos.z) * 8.0f);
            const float lo = EPS, hi_ = 8.0f - EPS;
            cp.x = gmin(gmax(cp.x, lo), hi_); cp.y = gmin(gmax(cp.y, lo), hi_); cp.z = gmin(gmax(cp.z, lo), hi_);
            int refracted;
            if (step_chunk(c, ts, pos, t, rayDir, &inv, &cp, ignoreFirst, maxDepth, hitNormal, vox,
                           colorAdd, colorMult, &refracted, hi)) {
                *rayPos = vadd(V((float)pos.x, (float)pos.y, (float)pos.z), vmuls(cp, INV_CHUNK));
                return 1;
            }
            if (c->capped) return 0;
            if (refracted) {
                *rayPos = vadd(V((float)pos.x, (float)pos.y, (float)pos.z), vmuls(cp, INV_CHUNK));
                init_dda(*rayDir, inv, *rayPos, &pos, &delta, &step, &side);
                lastSide = V(0.0f, 0.0f, 0.0f);
            }
        } else if (!requested && st != 0) {
            store_u8((uint8_t*)&m->state[t], 3);
            requested = 1;
        }
        lastSide = side;
        iter_dda(delta, step, &side, &pos, hitNormal);
        ignoreFirst = 0;
    }
    return 0;
}

static v3 sky_color(v3 bot, v3 top, v3 dir)
{
    /* voxelShared.comp:289-295, gradient branch; mix(x,y,a) = x*(1-a) + y*a (D12) */
    float a = dir.y * 0.5f + 1.0f;
    return V(bot.x * (1.0f - a) + top.x * a, bot.y * (1.0f - a) + top.y * a, bot.z * (1.0f - a) + top.z * a);
}

/* ---------------------------------------------------------------- lighting */

typedef struct lctx {
    ctx base;
    const dno_light_params* p;
    v3 sunDir, ambient, camPos, skyBot, skyTop;
    int firstSample;
    int rngSin;
    int persist;
    uint32_t key;           /* mode B per-voxel key */
    uint32_t sample;        /* current diffuse sample index */
    iv3 mapPos;
    uint8_t* vis;
} lctx;

static inline void ts_fresh(lctx* L, tstate* ts)
{
    if (!L->persist) { ts->lastVoxID = 255u; ts->lastVoxRefract = 1.0f; }
}

/* specular_ray, voxelLighting.comp:83-146 */
static void specular_ray(lctx* L, tstate* ts, v3 rayPos, v3 rayDir, v3 albedo, uint32_t reflectType, v3* color)
{
    ctx* c = &L->base;
    const dno_light_params* p = L->p;
    v3 lastPos = rayPos;
    v3 mult = albedo;
    voxel hv; memset(&hv, 0, sizeof(hv));
    ts_fresh(L, ts);
    for (uint32_t i = 0; i < p->specBounceLimit; i++) {
        v3 cadd; float cmul; v3 tn = V(0.0f, 0.0f, 0.0f); hitinfo hi;
        v3 inv = V(1.0f / rayDir.x, 1.0f / rayDir.y, 1.0f / rayDir.z);
        if (step_map(c, ts, &rayDir, inv, &rayPos, 1, -1.0f, &tn, &hv, &cadd, &cmul, &hi)) {
            /* visible propagation (D4: the lit chunk was visible when requested) */
            iv3 hp = {f2i(truncf(rayPos.x)), f2i(truncf(rayPos.y)), f2i(truncf(rayPos.z))};
            if (in_map(c->m, hp)) store_u8(&L->vis[map_index(c->m, hp)], 1);
            v3 a = vfloor(vmuls(rayPos, 8.0f)), b = vfloor(vmuls(lastPos, 8.0f));
            v3 d = vabs(vsub(a, b));
            if (dot3(d, d) <= 1.0f) return;
            const dno_material* hm = &c->mats[hv.material];
            hv.diff = vmuls(hv.diff, 1.0f - hm->specular);
            if (hm->emissive) {
                color->x = color->x + ((hv.albedo.x * c->emissive * cmul + cadd.x) * mult.x) * albedo.x;
                color->y = color->y + ((hv.albedo.y * c->emissive * cmul + cadd.y) * mult.y) * albedo.y;
                color->z = color->z + ((hv.albedo.z * c->emissive * cmul + cadd.z) * mult.z) * albedo.z;
                return;
            } else {
                v3 hc = vmul(hv.diff, hv.albedo);
                color->x = color->x + (hc.x * cmul + cadd.x) * mult.x;
                color->y = color->y + (hc.y * cmul + cadd.y) * mult.y;
                color->z = color->z + (hc.z * cmul + cadd.z) * mult.z;
                if (hm->specular == 0.0f) return;
                mult.x = mult.x * (hv.albedo.x * cmul * hm->specular);
                mult.y = mult.y * (hv.albedo.y * cmul * hm->specular);
                mult.z = mult.z * (hv.albedo.z * cmul * hm->specular);
                reflectType = hm->reflectType;
                lastPos = rayPos;
                rayDir = vreflect(rayDir, hv.normal);
            }
        } else if (dot3(rayDir, L->sunDir) > 0.99f) {
            color->x = color->x + (c->sunStrength.x * cmul + cadd.x);
            color->y = color->y + (c->sunStrength.y * cmul + cadd.y);
            color->z = color->z + (c->sunStrength.z * cmul + cadd.z);
            return;
        } else {
            v3 s = (reflectType == 1u) ? sky_color(L->skyBot, L->skyTop, rayDir) : c->sunStrength;
            color->x = color->x + (s.x * cmul + cadd.x) * mult.x;
            color->y = color->y + (s.y * cmul + cadd.y) * mult.y;
            color->z = color->z + (s.z * cmul + cadd.z) * mult.z;
            return;
        }
    }
}

/* diffuse_ray, voxelLighting.comp:149-203 */
static void diffuse_ray(lctx* L, tstate* ts, v3 normal, v3 rayPos, const voxel* initial, float seed, v3* color)
{
    ctx* c = &L->base;
    const dno_light_params* p = L->p;
    voxel hv = *initial;
    v3 hitNormal = normal;
    const dno_material* hm = &c->mats[initial->material];
    v3 nc = V(1.0f, 1.0f, 1.0f);
    v3 lastPos = rayPos;
    v3 lastDir = V(0.0f, 0.0f, 0.0f);
    ts_fresh(L, ts);
    for (uint32_t i = 0; i < p->diffuseBounceLimit; i++) {
        v3 dir;
        int lobe = 0;
        if (i > 0) {
            float r = L->rngSin ? srand1(seed + (float)p->diffuseBounceLimit + (float)i)
                                : hrand(L->key, 2u, (L->sample * 16u + i) << 8);
            lobe = (r + 1.0f) * 0.5f < hm->specular;
        }
        if (lobe) {
            v3 rs = L->rngSin ? sphere_sin(p->time + (float)i) : sphere_hash(L->key, 3u, L->sample * 16u + i);
            dir = vnormalize(vadd(vmuls(vreflect(lastDir, hitNormal), (float)hm->shininess), rs));
        } else if (L->firstSample) {
            dir = vadds(vnormalize(hitNormal), EPS);
        } else {
            v3 rs = L->rngSin ? sphere_sin(seed + (float)i) : sphere_hash(L->key, 1u, L->sample * 16u + i);
            dir = vadds(vnormalize(vadd(hitNormal, rs)), EPS);
        }
        v3 cadd; float cmul; v3 tn = V(0.0f, 0.0f, 0.0f); hitinfo hi;
        v3 inv = V(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
        int hit = step_map(c, ts, &dir, inv, &rayPos, 1, -1.0f, &tn, &hv, &cadd, &cmul, &hi);
        hitNormal = hv.normal;
        hm = &c->mats[hv.material];
        if (hit) {
            v3 a = vfloor(vmuls(lastPos, 8.0f)), b = vfloor(vmuls(rayPos, 8.0f));
            v3 d = vabs(vsub(a, b));
            if (dot3(d, d) < 1.0f) return;
            if (hm->emissive) {
                color->x = color->x + nc.x * (hv.albedo.x * c->emissive * cmul + cadd.x);
                color->y = color->y + nc.y * (hv.albedo.y * c->emissive * cmul + cadd.y);
                color->z = color->z + nc.z * (hv.albedo.z * c->emissive * cmul + cadd.z);
                return;
            }
            nc.x = nc.x * (hv.albedo.x * cmul + cadd.x);
            nc.y = nc.y * (hv.albedo.y * cmul + cadd.y);
            nc.z = nc.z * (hv.albedo.z * cmul + cadd.z);
        } else {
            float k = gmax(dot3(dir, L->sunDir), 0.0f);
            color->x = color->x + (nc.x * k * c->sunStrength.x * cmul + cadd.x);
            color->y = color->y + (nc.y * k * c->sunStrength.y * cmul + cadd.y);
            color->z = color->z + (nc.z * k * c->sunStrength.z * cmul + cadd.z);
            return;
        }
        lastDir = dir;
    }
}

/* one shadow ray (voxelLighting.comp:65-80); adds sunStrength*colorMult + colorAdd on a miss */
static void shadow_ray(lctx* L, tstate* ts, v3 rayPos, v3 dir, v3* color)
{
    ctx* c = &L->base;
    voxel hv; v3 cadd; float cmul; v3 tn = V(0.0f, 0.0f, 0.0f); hitinfo hi;
    ts_fresh(L, ts);
    v3 inv = V(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    if (!step_map(c, ts, &dir, inv, &rayPos, 1, -1.0f, &tn, &hv, &cadd, &cmul, &hi)) {
        color->x = color->x + (c->sunStrength.x * cmul + cadd.x);
        color->y = color->y + (c->sunStrength.y * cmul + cadd.y);
        color->z = color->z + (c->sunStrength.z * cmul + cadd.z);
    }
}

#define DNO_REFERENCE_SHADOW 4u   /* pinning only: one jittered shadow ray per sample (voxelLighting.comp:65-80, 260) */

/* voxelLighting.comp:207-288 for one voxel; returns 0 if voxNum is past the chunk's voxels */
static int light_voxel(lctx* L, uint32_t tile, uint32_t voxNum, float outDiff[3], float outSpec[3])
{
    ctx* c = &L->base;
    const dno_map* m = c->m;
    const dno_light_params* p = L->p;
    const orec* r = &m->rec[tile];
    iv3 cp;
    if (!vox_select(r, voxNum, &cp)) return 0;
    iv3 mp = {(int32_t)(tile % m->sx), (int32_t)((tile / m->sx) % m->sy), (int32_t)(tile / ((uint64_t)m->sx * m->sy))};
    L->mapPos = mp;
    voxel tv; decompress(r, voxNum, &tv);
    const dno_material* tm = &c->mats[tv.material];
    uint32_t ns = r->samples < p->maxDiffuse ? r->samples : p->maxDiffuse;
    float indirect = (float)ns;
    L->firstSample = (indirect == 0.0f);
    uint32_t gx = (uint32_t)(mp.x * 8 + cp.x), gy = (uint32_t)(mp.y * 8 + cp.y), gz = (uint32_t)(mp.z * 8 + cp.z);
    uint32_t gidx = gx + (m->sx * 8u) * (gy + (m->sy * 8u) * gz);
    uint32_t tb; memcpy(&tb, &p->time, 4);
    L->key = rng_key(tb, p->mapId, gidx);

    v3 rayPos;
    rayPos.x = INV_CHUNK * (float)cp.x + (float)mp.x + HALF_INV_CHUNK;
    rayPos.y = INV_CHUNK * (float)cp.y + (float)mp.y + HALF_INV_CHUNK;
    rayPos.z = INV_CHUNK * (float)cp.z + (float)mp.z + HALF_INV_CHUNK;
    const float off = HALF_INV_CHUNK - EPS;
    rayPos = vadd(rayPos, vmuls(tv.normal, off));

    v3 spec = V(0.0f, 0.0f, 0.0f), diff = V(0.0f, 0.0f, 0.0f);
    tstate ts = {255u, 1.0f};
    uint32_t K = p->K;
    v3 viewDir = vsub(rayPos, L->camPos);
    if (tm->specular > 0.0f && dot3(viewDir, tv.normal) < 0.0f && tm->reflectType <= 1u) {
        v3 refl = vreflect(vnormalize(viewDir), tv.normal);
        for (uint32_t k = 0; k < K; k++) {
            v3 P = V(p->spherePts[k][0], p->spherePts[k][1], p->spherePts[k][2]);
            v3 sd = vadds(vnormalize(vadd(vmuls(refl, (float)tm->shininess), P)), EPS);
            specular_ray(L, &ts, rayPos, sd, tv.albedo, tm->reflectType, &spec);
        }
        spec = vdivs(spec, (float)K);
    }
    if (tm->specular < 1.0f) {
        v3 direct = V(0.0f, 0.0f, 0.0f);
        int refShadow = (p->flags & DNO_REFERENCE_SHADOW) != 0;
        if (!refShadow) {
            /* D8: K fixed shadow rays traced once, averaged */
            v3 sum = V(0.0f, 0.0f, 0.0f);
            if (L->firstSample) {
                shadow_ray(L, &ts, rayPos, vadds(L->sunDir, EPS), &sum);
                direct = vdivs(sum, 1.0f);
            } else {
                for (uint32_t k = 0; k < K; k++) {
                    v3 P = V(p->spherePts[k][0], p->spherePts[k][1], p->spherePts[k][2]);
                    v3 d = vadds(vnormalize(vadd(vmuls(L->sunDir, p->shadowSoftness), P)), EPS);
                    shadow_ray(L, &ts, rayPos, d, &sum);
                }
                direct = vdivs(sum, (float)K);
            }
        }
        for (uint32_t i = 0; i < p->numDiffuse; i++) {
            L->sample = i;
            diff = vadd(diff, L->ambient);
            diffuse_ray(L, &ts, vadds(tv.normal, EPS), rayPos, &tv, p->time * (float)(i + 1u), &diff);
            if (refShadow) {
                v3 d;
                if (L->firstSample) d = vadds(L->sunDir, EPS);
                else {
                    v3 rs = L->rngSin ? sphere_sin(p->time * (float)(i + 1u + p->numDiffuse))
                                      : sphere_hash(L->key, 4u, i);
                    d = vadds(vnormalize(vadd(vmuls(L->sunDir, p->shadowSoftness), rs)), EPS);
                }
                shadow_ray(L, &ts, rayPos, d, &diff);
            } else {
                diff = vadd(diff, direct);
            }
        }
        float den = indirect + (float)p->numDiffuse;
        diff.x = (tv.diff.x * indirect + diff.x) / den;
        diff.y = (tv.diff.y * indirect + diff.y) / den;
        diff.z = (tv.diff.z * indirect + diff.z) / den;
    }
    /* clamp (voxelLighting.comp:267-268) */
    outSpec[0] = gmin(gmax(spec.x, 0.0f), 1.0f); outSpec[1] = gmin(gmax(spec.y, 0.0f), 1.0f); outSpec[2] = gmin(gmax(spec.z, 0.0f), 1.0f);
    outDiff[0] = gmin(gmax(diff.x, 0.0f), 1.0f); outDiff[1] = gmin(gmax(diff.y, 0.0f), 1.0f); outDiff[2] = gmin(gmax(diff.z, 0.0f), 1.0f);
    c->c.litVoxels++;
    return 1;
}

static void lctx_init(lctx* L, dno_map* m, const dno_material* mats, const dno_light_params* p)
{
    memset(L, 0, sizeof(*L));
    L->base.m = m;
    L->base.mats = mats;
    L->base.sunStrength = V(p->sunStrength[0], p->sunStrength[1], p->sunStrength[2]);
    L->base.emissive = p->emissiveStrength;
    L->base.refraction = 0;   /* voxelLighting.comp:209 */
    L->p = p;
    L->sunDir = V(p->sunDir[0], p->sunDir[1], p->sunDir[2]);
    L->ambient = V(p->ambient[0], p->ambient[1], p->ambient[2]);
    L->camPos = V(p->camPos[0], p->camPos[1], p->camPos[2]);
    L->skyBot = V(p->skyBot[0], p->skyBot[1], p->skyBot[2]);
    L->skyTop = V(p->skyTop[0], p->skyTop[1], p->skyTop[2]);
    L->rngSin = (p->flags & DNO_RNG_SIN) != 0;
    L->persist = (p->flags & DNO_PERSIST_TRANSPARENCY) != 0;
    L->vis = m->vis;
}

static void add_counters(dno_counters* d, const dno_counters* s)
{
    d->rays += s->rays; d->primary += s->primary; d->outerSteps += s->outerSteps;
    d->chunksEntered += s->chunksEntered; d->innerSteps += s->innerSteps; d->hits += s->hits;
    d->litVoxels += s->litVoxels;
    d->degenerate += s->degenerate;
}

static dno_light_params fix_params(const dno_light_params* p)
{
    dno_light_params q = *p;
    if (q.K > 64) q.K = 64;
    if (q.K < 1) q.K = 1;
    if (!q.useSpherePoints) dno_sphere_points(q.K, q.spherePts);
    return q;
}

void dno_light(dno_map* m, const dno_material* mats, const dno_light_params* p0, int nthreads)
{
    dno_light_params p = fix_params(p0);
    uint32_t nreq = m->nreq;
    float* od = (float*)malloc(sizeof(float) * 3 * 32 * (size_t)(nreq ? nreq : 1));
    float* os = (float*)malloc(sizeof(float) * 3 * 32 * (size_t)(nreq ? nreq : 1));
    uint8_t* ok = (uint8_t*)calloc((size_t)32 * (nreq ? nreq : 1), 1);
    dno_counters total; memset(&total, 0, sizeof(total));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        lctx L; lctx_init(&L, m, mats, &p);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int64_t q = 0; q < (int64_t)nreq; q++) {
            uint32_t w = m->req[q];
            uint32_t tile = w >> 4, group = w & 15u;
            if (m->state[tile] != 2) continue;
            for (uint32_t lane = 0; lane < 32; lane++) {
                uint32_t vn = lane + group * 32u;
                ok[q * 32 + lane] = (uint8_t)light_voxel(&L, tile, vn, &od[(q * 32 + lane) * 3], &os[(q * 32 + lane) * 3]);
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        add_counters(&total, &L.base.c);
    }
    /* commit (D1) and sample counts (D2) */
    for (uint32_t q = 0; q < nreq; q++) {
        uint32_t tile = m->req[q] >> 4, group = m->req[q] & 15u;
        if (m->state[tile] != 2) continue;
        orec* r = &m->rec[tile];
        for (uint32_t lane = 0; lane < 32; lane++) {
            if (!ok[q * 32 + lane]) continue;
            uint32_t vn = lane + group * 32u;
            memcpy(r->diff[vn], &od[(q * 32 + lane) * 3], sizeof(float) * 3);
            memcpy(r->spec[vn], &os[(q * 32 + lane) * 3], sizeof(float) * 3);
        }
        if (group == 0 && ok[q * 32]) r->samples++;
    }
    add_counters(&m->ctr, &total);
    free(od); free(os); free(ok);
}

void dno_light_requests(dno_map* m, const dno_material* mats, const dno_light_params* p0,
                        const uint32_t* reqIdx, uint32_t n, float* out_diff, float* out_spec,
                        uint8_t* valid, int nthreads)
{
    dno_light_params p = fix_params(p0);
    dno_counters total; memset(&total, 0, sizeof(total));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        lctx L; lctx_init(&L, m, mats, &p);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t j = 0; j < (int64_t)n; j++) {
            uint32_t w = m->req[reqIdx[j]];
            uint32_t tile = w >> 4, group = w & 15u;
            for (uint32_t lane = 0; lane < 32; lane++) {
                valid[j * 32 + lane] = 0;
                if (m->state[tile] != 2) continue;
                valid[j * 32 + lane] = (uint8_t)light_voxel(&L, tile, lane + group * 32u,
                                                            &out_diff[(j * 32 + lane) * 3], &out_spec[(j * 32 + lane) * 3]);
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        add_counters(&total, &L.base.c);
    }
    add_counters(&m->ctr, &total);
}

/* -------------------------------------------------------------------- draw */

static void mat4_mul(const float A[4][4], const float B[4][4], float C[4][4])
{
    /* C = A * B, column-major m[col][row]; sum over k in order */
    for (int col = 0; col < 4; col++)
        for (int row = 0; row < 4; row++)
            C[col][row] = A[0][row] * B[col][0] + A[1][row] * B[col][1] + A[2][row] * B[col][2] + A[3][row] * B[col][3];
}

static inline float gpow(float x, float y) { return powf(x, y); }

/* Texel of floor coordinate f under GL_REPEAT on a texture n texels wide. */
static uint32_t repeat_texel(float f, uint32_t n)
{
    int k = (int)f % (int)n;
    return (uint32_t)(k < 0 ? k + (int)n : k);
}

/* GL_LINEAR sample with GL_REPEAT at texture coordinate (s, t): the OpenGL 4.3 formula (section 8.14.2)
 * u = s*w - 1/2, i0 = wrap(floor(u)), i1 = wrap(floor(u) + 1), alpha = u - floor(u) (same along t), then
 * (1-a)(1-b) T00 + a(1-b) T10 + (1-a)b T01 + ab T11 in that order.  The reference samples its raster
 * textures this way (main.c:313-322 set GL_LINEAR; the wrap stays at its GL_REPEAT default;
 * voxelDraw.comp:28, 89).  C floats per texel, the first n returned. */
static void raster_sample(const float* tex, uint32_t w, uint32_t h, int C, int n, float s, float t, float* out)
{
    float u = s * (float)w - 0.5f, v = t * (float)h - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    uint32_t i0 = repeat_texel(fu, w), j0 = repeat_texel(fv, h);
    uint32_t i1 = i0 + 1u == w ? 0u : i0 + 1u, j1 = j0 + 1u == h ? 0u : j0 + 1u;
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    for (int k = 0; k < n; k++)
        out[k] = w00 * tex[((size_t)j0 * w + i0) * C + k] + w10 * tex[((size_t)j0 * w + i1) * C + k]
               + w01 * tex[((size_t)j1 * w + i0) * C + k] + w11 * tex[((size_t)j1 * w + i1) * C + k];
}

/* background_color (voxelDraw.comp:24-30): the sky when no raster depth is tested, else the raster colour */
static v3 background(const dno_draw_params* p, float maxDepth, float texS, float texT, v3 skyBot, v3 skyTop, v3 dir)
{
    if (maxDepth < 0.0f) {
        v3 s = sky_color(skyBot, skyTop, dir);
        return V(gpow(s.x, 2.2f), gpow(s.y, 2.2f), gpow(s.z, 2.2f));
    }
    float rc[3];
    raster_sample(p->rasterColor, p->rasterColorW, p->rasterColorH, 4, 3, texS, texT, rc);
    return V(rc[0], rc[1], rc[2]);
}

void dno_draw(dno_map* m, const dno_material* mats, const dno_draw_params* p,
              float* color, uint32_t* hitOut, uint8_t* faceOut, int nthreads)
{
    float M[4][4];
    mat4_mul(p->invCenteredView, p->invProj, M);
    /* invView * (0,0,0,1) */
    v3 origin = V(p->invView[0][0] * 0.0f + p->invView[1][0] * 0.0f + p->invView[2][0] * 0.0f + p->invView[3][0] * 1.0f,
                  p->invView[0][1] * 0.0f + p->invView[1][1] * 0.0f + p->invView[2][1] * 0.0f + p->invView[3][1] * 1.0f,
                  p->invView[0][2] * 0.0f + p->invView[1][2] * 0.0f + p->invView[2][2] * 0.0f + p->invView[3][2] * 1.0f);
    uint32_t W = p->width, H = p->height;
    uint64_t npix = p->pixels ? p->npixels : (uint64_t)W * H;
    uint32_t limW = p->truncate16 ? (W / 16u) * 16u : W, limH = p->truncate16 ? (H / 16u) * 16u : H;
    v3 skyBot = V(p->skyBot[0], p->skyBot[1], p->skyBot[2]), skyTop = V(p->skyTop[0], p->skyTop[1], p->skyTop[2]);
    v3 mapMax = V((float)m->sx, (float)m->sy, (float)m->sz);
    dno_counters total; memset(&total, 0, sizeof(total));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        ctx c; memset(&c, 0, sizeof(c));
        c.m = m; c.mats = mats; c.sunStrength = V(p->sunStrength[0], p->sunStrength[1], p->sunStrength[2]);
        c.emissive = p->emissiveStrength; c.refraction = 1;   /* voxelDraw.comp:65 */
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (int64_t j = 0; j < (int64_t)npix; j++) {
            uint32_t pix = p->pixels ? p->pixels[j] : (uint32_t)j;
            uint32_t x = pix % W, y = pix / W;
            float* out = &color[j * 4];
            hitOut[j] = 0xFFFFFFFFu; faceOut[j] = 6;
            if (x >= limW || y >= limH) { out[0] = out[1] = out[2] = 0.0f; out[3] = -1.0f; continue; }
            float sx = (float)x / (float)W * 2.0f - 1.0f;
            float sy = (float)y / (float)H * 2.0f - 1.0f;
            v3 rayPos = origin;
            c.orgRayPos = rayPos;
            v3 rd = V(M[0][0] * sx + M[1][0] * sy + M[2][0] * 0.0f + M[3][0] * 1.0f,
                      M[0][1] * sx + M[1][1] * sy + M[2][1] * 0.0f + M[3][1] * 1.0f,
                      M[0][2] * sx + M[1][2] * sy + M[2][2] * 0.0f + M[3][2] * 1.0f);
            v3 rayDir = vadds(vnormalize(rd), EPS);
            v3 inv = V(1.0f / rayDir.x, 1.0f / rayDir.y, 1.0f / rayDir.z);
            /* raster depth as a distance from the camera, voxelDraw.comp:86-101 (negative: not tested) */
            float maxDepth = -1.0f, texS = 0.0f, texT = 0.0f;
            if (p->compose) {
                texS = (float)x / (float)p->rasterColorW;
                texT = (float)y / (float)p->rasterColorH;
                float d;
                raster_sample(p->rasterDepth, p->rasterDepthW, p->rasterDepthH, 1, 1, texS, texT, &d);
                maxDepth = d * 2.0f - 1.0f;
                if (maxDepth < 1.0f) {
                    float vs[4];
                    for (int r = 0; r < 4; r++)
                        vs[r] = p->invProj[0][r] * sx + p->invProj[1][r] * sy + p->invProj[2][r] * maxDepth + p->invProj[3][r] * 1.0f;
                    v3 vp = V(vs[0] / vs[3], vs[1] / vs[3], vs[2] / vs[3]);
                    maxDepth = sqrtf(dot3(vp, vp));
                } else {
                    maxDepth = -1.0f;
                }
            }
            /* intersect_AABB, voxelShared.comp:261-273 */
            v3 tMin = vmul(vsub(V(0.0f, 0.0f, 0.0f), rayPos), inv);
            v3 tMax = vmul(vsub(mapMax, rayPos), inv);
            v3 t1 = V(gmin(tMin.x, tMax.x), gmin(tMin.y, tMax.y), gmin(tMin.z, tMax.z));
            v3 t2 = V(gmax(tMin.x, tMax.x), gmax(tMin.y, tMax.y), gmax(tMin.z, tMax.z));
            float tNear = gmax(gmax(t1.x, t1.y), t1.z);
            float tFar = gmin(gmin(t2.x, t2.y), t2.z);
            v3 fc; float depth = -1.0f;
            if (tNear > tFar || tFar < 0.0f) {
                fc = background(p, maxDepth, texS, texT, skyBot, skyTop, rayDir);
            } else {
                if (tNear > 0.0f) rayPos = vadd(rayPos, vmuls(rayDir, tNear + EPS));
                /* normal_AABB, voxelShared.comp:276-284 */
                v3 cc = vmuls(vadd(V(0.0f, 0.0f, 0.0f), mapMax), 0.5f);
                v3 pp = vsub(rayPos, cc);
                v3 dd = vmuls(vsub(mapMax, V(0.0f, 0.0f, 0.0f)), 0.5f);
                const float bias = 1.0f + EPS;
                v3 q = vmuls(vdivv(pp, dd), bias);
                v3 hitNormal = vnormalize(V(truncf(q.x), truncf(q.y), truncf(q.z)));
                tstate ts = {255u, 1.0f};
                voxel fv; memset(&fv, 0, sizeof(fv));
                v3 cadd; float cmul; hitinfo hi;
                c.c.primary++;
                if (step_map(&c, &ts, &rayDir, inv, &rayPos, 0, maxDepth, &hitNormal, &fv, &cadd, &cmul, &hi)) {
                    iv3 mp = {f2i(floorf(rayPos.x)), f2i(floorf(rayPos.y)), f2i(floorf(rayPos.z))};
                    if (in_map(m, mp)) store_u8(&m->vis[map_index(m, mp)], 1);
                    v3 dv = vsub(rayPos, c.orgRayPos);
                    depth = sqrtf(dot3(dv, dv));
                    if (maxDepth > 0.0f && depth > maxDepth) {
                        /* the rasterised scene is in front (voxelDraw.comp:127-131): no voxel is reported */
                        fc = vadd(vmuls(background(p, maxDepth, texS, texT, skyBot, skyTop, rayDir), cmul), cadd);
                        depth = maxDepth;
                        goto store;
                    }
                    /* voxel_color, voxelDraw.comp:32-61 */
                    const dno_material* mt = &mats[fv.material];
                    v3 sp = vmuls(fv.spec, mt->specular);
                    v3 df = vmuls(fv.diff, 1.0f - mt->specular);
                    switch (p->viewMode) {
                    case 0: {
                        v3 solid;
                        if (mt->emissive) solid = vmuls(fv.albedo, c.emissive);
                        else solid = vadd(vmul(df, fv.albedo), sp);
                        fc = vadd(vmuls(solid, cmul), cadd);
                        break;
                    }
                    case 1: fc = fv.albedo; break;
                    case 2: fc = mt->emissive ? fv.albedo : df; break;
                    case 3: fc = mt->emissive ? fv.albedo : sp; break;
                    case 4: fc = vabs(fv.normal); break;
                    case 5: fc = vabs(hitNormal); break;
                    default: fc = V(0.0f, 0.0f, 0.0f); break;
                    }
                    uint32_t gx = (uint32_t)((int32_t)(hi.tile % m->sx) * 8 + hi.local.x);
                    uint32_t gy = (uint32_t)((int32_t)((hi.tile / m->sx) % m->sy) * 8 + hi.local.y);
                    uint32_t gz = (uint32_t)((int32_t)(hi.tile / ((uint64_t)m->sx * m->sy)) * 8 + hi.local.z);
                    hitOut[j] = gx + (m->sx * 8u) * (gy + (m->sy * 8u) * gz);
                    uint8_t f = 6;
                    if (hitNormal.x > 0.0f) f = 0; else if (hitNormal.x < 0.0f) f = 1;
                    else if (hitNormal.y > 0.0f) f = 2; else if (hitNormal.y < 0.0f) f = 3;
                    else if (hitNormal.z > 0.0f) f = 4; else if (hitNormal.z < 0.0f) f = 5;
                    faceOut[j] = f;
                } else {
                    fc = vadd(vmuls(background(p, maxDepth, texS, texT, skyBot, skyTop, rayDir), cmul), cadd);
                    depth = maxDepth;
                }
            }
        store:
            out[0] = gpow(fc.x, 0.4545f); out[1] = gpow(fc.y, 0.4545f); out[2] = gpow(fc.z, 0.4545f);
            out[3] = depth;
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        add_counters(&total, &c.c);
    }
    add_counters(&m->ctr, &total);
}

/* ---------------------------------------------------------------- exports */

uint32_t dno_num_requests(const dno_map* m) { return m->nreq; }
const uint32_t* dno_requests(const dno_map* m) { return m->req; }
uint32_t dno_frame_num(const dno_map* m) { return m->frameNum; }
void dno_get_counters(const dno_map* m, dno_counters* out) { *out = m->ctr; }
void dno_reset_counters(dno_map* m) { memset(&m->ctr, 0, sizeof(m->ctr)); }

void dno_export_tiles(const dno_map* m, uint8_t* state, uint8_t* vis, uint32_t* lastUsed)
{
    for (uint64_t t = 0; t < m->ntiles; t++) {
        if (state) state[t] = m->state[t];
        if (vis) vis[t] = m->vis[t];
        if (lastUsed) lastUsed[t] = m->lastUsed[t];
    }
}

static uint32_t global_index(const dno_map* m, uint64_t tile, iv3 cp)
{
    uint32_t gx = (uint32_t)((tile % m->sx) * 8 + (uint32_t)cp.x);
    uint32_t gy = (uint32_t)(((tile / m->sx) % m->sy) * 8 + (uint32_t)cp.y);
    uint32_t gz = (uint32_t)((tile / ((uint64_t)m->sx * m->sy)) * 8 + (uint32_t)cp.z);
    return gx + (m->sx * 8u) * (gy + (m->sy * 8u) * gz);
}

uint64_t dno_export_lighting(const dno_map* m, uint32_t* index, float* diff, float* spec)
{
    uint64_t n = 0;
    for (uint64_t t = 0; t < m->ntiles; t++) {
        if (m->state[t] != 2) continue;
        const orec* r = &m->rec[t];
        for (uint32_t v = 0; v < r->nvox; v++) {
            if (index) {
                iv3 cp; vox_select(r, v, &cp);
                index[n] = global_index(m, t, cp);
                memcpy(&diff[n * 3], r->diff[v], 12);
                memcpy(&spec[n * 3], r->spec[v], 12);
            }
            n++;
        }
    }
    return n;
}

void dno_export_samples(const dno_map* m, uint32_t* samples)
{
    for (uint64_t t = 0; t < m->ntiles; t++) samples[t] = (m->state[t] == 2) ? m->rec[t].samples : 0u;
}

void dno_import_lighting(dno_map* m, uint64_t n, const uint32_t* index, const float* diff, const float* spec)
{
    uint32_t VX = m->sx * 8u, VY = m->sy * 8u;
    for (uint64_t i = 0; i < n; i++) {
        uint32_t g = index[i];
        uint32_t gx = g % VX, gy = (g / VX) % VY, gz = g / (VX * VY);
        iv3 mp = {(int32_t)(gx / 8), (int32_t)(gy / 8), (int32_t)(gz / 8)};
        iv3 cp = {(int32_t)(gx % 8), (int32_t)(gy % 8), (int32_t)(gz % 8)};
        if (!in_map(m, mp)) continue;
        uint32_t t = map_index(m, mp);
        if (m->state[t] != 2) continue;
        orec* r = &m->rec[t];
        if (!vox_exists(r, cp)) continue;
        uint32_t rank = vox_rank(r, cp);
        memcpy(r->diff[rank], &diff[i * 3], 12);
        memcpy(r->spec[rank], &spec[i * 3], 12);
    }
}

void dno_import_samples(dno_map* m, const uint32_t* samples)
{
    for (uint64_t t = 0; t < m->ntiles; t++) if (m->state[t] == 2) m->rec[t].samples = samples[t];
}

void dno_import_state(dno_map* m, const dno_handle* cpuMap, const dno_chunk* chunks, const dno_material* mats,
                      const uint8_t* state, const uint8_t* vis, uint32_t frameNum)
{
    for (uint64_t t = 0; t < m->ntiles; t++) {
        uint8_t st = state[t];
        if (st == 2) {
            if (m->state[t] != 2 && cpuMap[t].flag) rec_load(&m->rec[t], &chunks[cpuMap[t].chunkIndex], mats);
            if (!cpuMap[t].flag) st = 0;
        } else if (m->state[t] == 2) {
            rec_free(&m->rec[t]);
        }
        m->state[t] = st;
        m->vis[t] = vis ? vis[t] : 0;
        m->touch[t] = 0;
    }
    m->frameNum = frameNum;
}

void dno_set_requests(dno_map* m, const uint32_t* words, uint32_t n)
{
    m->nreq = 0;
    for (uint32_t i = 0; i < n; i++) push_req(m, words[i]);
}
