/*
 * dn_oracle.h -- CPU oracle for the DoonEngine per-voxel lighting + draw path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * GLSL compute shaders (assets/shaders/voxelShared.comp, voxelLighting.comp,
 * voxelDraw.comp) and of the host-side packing / sync logic in
 * src/DoonEngine/voxel.c.  It is the oracle that the CUDA path is compared
 * against and the timed CPU baseline; the product library never links,
 * loads or calls it.
 *
 * Parity status: pinned.  The reference has no tests and its hot path exists
 * only as GLSL, which cannot run on these machines through a graphics API.
 * The host-side pieces (voxel codec, chunk packing, edit API, camera, CPU
 * picking ray, .voxvol codec) are pinned against the reference's own C
 * compiled from its sources (oracle/ref/dnref_shim.c); the shader
 * transcription is pinned by running the reference's shader source itself
 * on the CPU, translated to C++ (oracle/ref/glsl_to_cpp.py, glsl_shim.hpp,
 * pin_harness.cpp), in this oracle's reference-faithful modes
 * (DNO_RNG_SIN | DNO_PERSIST_TRANSPARENCY | DNO_REFERENCE_SHADOW with the
 * shader's 15-point table).  Only the sine both sides use is this project's
 * deterministic sine rather than a GPU's.
 *
 * Deterministic semantics where the reference races or is undefined
 * (numbered D1..D16, each applied identically here and in the kernels):
 *   D1  lighting reads the previous frame's committed lighting; results are
 *       committed after the whole launch (reference reads/writes in place,
 *       voxelLighting.comp:113,122 vs 276-278).
 *   D2  the per-chunk sample count is read once per launch and incremented
 *       after it (voxelLighting.comp:224 vs 284-285).
 *   D3  FP32 lighting accumulators (reference quantises to 8/16 bit,
 *       voxelLighting.comp:266-278).
 *   D4  visible / requested / touched are per-tile bytes written with
 *       idempotent stores; visible is cleared when a chunk is taken into the
 *       lighting request list; "touched" (lastUsed = 0) is recorded when a
 *       ray enters a loaded chunk (voxelShared.comp:143-144, 464;
 *       voxelDraw.comp:121; voxelLighting.comp:104-105, 281).
 *   D5  RNG mode B (default): integer hash of (map, voxel, seed, stream,
 *       index); mode A: the reference's fract(sin(s)*43758.5453) with a
 *       project-written deterministic sine (voxelLighting.comp:29-57).
 *   D6  rand_unit_sphere gives up after 64 tries and returns (0,0,0)
 *       (voxelLighting.comp:47-57 loops without bound).
 *   D7  the draw covers every pixel; a flag emulates the reference's
 *       w/16 x h/16 dispatch truncation (voxel.c:879).
 *   D8  direct light = mean of K fixed shadow rays along
 *       normalize(sunDir*softness + P_k) (P_k: K-point golden-angle sphere),
 *       traced once per voxel and added once per diffuse sample; on the first
 *       sample one ray along sunDir+EPS (voxelLighting.comp:65-80).  Specular
 *       uses the same K points (voxelLighting.comp:23, 244-250).
 *   D9  emissive hits are scaled by a volume-wide emissive strength
 *       (1.0 = reference; voxelLighting.comp:117,189; voxelDraw.comp:44).
 *   D10 device voxels are two 32-bit words: the reference's packed normal
 *       word (material<<24 | n.x<<16 | n.y<<8 | n.z) and the linearised albedo
 *       word (voxel.c:1438-1452).
 *   D11 no FMA contraction; IEEE division and square root; GLSL built-ins
 *       (min, max, clamp, mix, reflect, refract, normalize, sign, fract) follow
 *       their specification formulas.
 *   D12 the sky gradient keeps the reference's y*0.5+1 parameter
 *       (voxelShared.comp:294).
 *   D13 refraction only in the draw (voxelDraw.comp:65).  The transparency
 *       state (lastVoxID / lastVoxRefract, voxelShared.comp:321-325) starts
 *       fresh for every primary ray and every lighting ray job (one shadow
 *       ray, one specular ray with its bounces, one diffuse path with its
 *       bounces); the reference carries it across all rays of one shader
 *       invocation, which makes results depend on ray order.  Mode
 *       DNO_PERSIST_TRANSPARENCY restores the reference behaviour (pinning
 *       only).
 *   D14 face code from the hit normal: 0 +x, 1 -x, 2 +y, 3 -y, 4 +z, 5 -z,
 *       6 none; hit index = global voxel coordinate x + X*(y + Y*z) in voxels,
 *       0xFFFFFFFF on a miss.
 *   D15 the GLSL <= multi-axis tie step (voxelShared.comp:313) is
 *       authoritative; the CPU picking ray keeps its own strict < (voxel.c:1241).
 *   D16 a traversal segment (one step_map call) that has visited
 *       256 * (sx + sy + sz) + 4096 cells (outer plus inner iterations, at
 *       most 2^23) ends as a miss.  Ordinary rays leave the map long before;
 *       a zero or NaN direction component makes a side distance NaN
 *       (0 * inf) after one step, after which the reference's loop
 *       (voxelShared.comp:339, 435) would never end.
 *   D18 LRU residency (dno_set_lru): the reference's node buffer decides
 *       loads, unloads and growth in its tile order (voxel.c:1491-1695); a
 *       chunk unloaded later in the same sync keeps its requests, which
 *       light nothing (the reference would light the slots' new data); a
 *       reload packs the chunk again; with no node the sort does not run.
 *       Unpinned: the reference's allocator touches OpenGL on every path.
 */
#ifndef DN_ORACLE_H
#define DN_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- layouts of the reference's public CPU-side structs (voxel.h:35-94) ---- */

typedef struct dno_cvoxel { uint32_t normal, albedo; } dno_cvoxel;      /* DNcompressedVoxel */

typedef struct dno_chunk {                                               /* DNchunk */
    int32_t pos[3];
    uint8_t updated;
    uint32_t numVoxels;
    uint32_t numVoxelsGpu;
    dno_cvoxel voxels[8][8][8];   /* [x][y][z] */
} dno_chunk;

typedef struct dno_handle { uint8_t flag; uint32_t chunkIndex; } dno_handle;   /* DNchunkHandle */

typedef struct dno_material {                                            /* DNmaterial (std140, 32 B) */
    float padding[2];
    uint32_t emissive;
    float opacity;
    float refractIndex;
    float specular;
    uint32_t reflectType;
    uint32_t shininess;
} dno_material;

/* ---- packed chunk (restatement of _DN_chunk_to_gpu, voxel.c:1397-1461) ---- */
typedef struct dno_packed {
    uint32_t mask[16];
    uint32_t partial[3];
    uint32_t nvox;
    uint32_t vox[512][2];         /* [normal word, linear albedo word] */
} dno_packed;

void dno_pack_chunk(const dno_chunk* chunk, const dno_material* materials, dno_packed* out);

/* voxel codec restatements (voxel.c:1289-1316) */
void dno_compress_voxel(uint8_t material, const float normal[3], const uint8_t albedo[3], dno_cvoxel* out);
void dno_decompress_voxel(dno_cvoxel v, uint8_t* material, float normal[3], uint8_t albedo[3]);

/* ---- oracle map state: the device-side state of one volume ---- */
typedef struct dno_map dno_map;

dno_map* dno_create(uint32_t sx, uint32_t sy, uint32_t sz);
void dno_destroy(dno_map* m);

/* modes */
#define DNO_RNG_HASH 0              /* D5 mode B */
#define DNO_RNG_SIN  1              /* D5 mode A */
#define DNO_PERSIST_TRANSPARENCY 2  /* D13: carry lastVoxID across rays (pinning only) */

typedef struct dno_light_params {
    float sunDir[3];          /* already normalised by the caller (voxel.c:942) */
    float sunStrength[3];
    float ambient[3];
    float camPos[3];
    float skyBot[3], skyTop[3];
    float shadowSoftness;
    float time;               /* latched time (voxel.c:886-887) */
    float emissiveStrength;   /* D9 */
    uint32_t numDiffuse, maxDiffuse;
    uint32_t diffuseBounceLimit, specBounceLimit;
    uint32_t K;               /* fixed direct / specular ray count (D8), <= 64 */
    uint32_t flags;           /* DNO_RNG_* | DNO_PERSIST_TRANSPARENCY */
    uint32_t mapId;           /* hash key component (D5) */
    uint32_t useSpherePoints; /* 1: use spherePts below verbatim (K entries) */
    float spherePts[64][3];
} dno_light_params;

typedef struct dno_draw_params {
    float invView[4][4];          /* column-major m[col][row] */
    float invCenteredView[4][4];
    float invProj[4][4];
    uint32_t width, height;
    uint32_t viewMode;
    uint32_t truncate16;          /* D7 */
    float sunStrength[3];
    float skyBot[3], skyTop[3];
    float emissiveStrength;
    /* pixel subset (NULL = all pixels): list of pixel indices y*width+x */
    const uint32_t* pixels;
    uint32_t npixels;
    /* raster composition (voxelDraw.comp:86-101, 127-136) when compose is 1: colour RGBA (4 floats per
     * texel, alpha unused) and window depth (1 float per texel), texel (i, j) at [j * w + i]; sampled
     * GL_LINEAR with GL_REPEAT at texture coordinate (x / colorW, y / colorH) */
    uint32_t compose;
    const float* rasterColor;
    const float* rasterDepth;
    uint32_t rasterColorW, rasterColorH, rasterDepthW, rasterDepthH;
} dno_draw_params;

typedef struct dno_counters {
    uint64_t rays;            /* step_map calls (all kinds) */
    uint64_t primary;         /* primary rays that entered step_map */
    uint64_t outerSteps;      /* chunk cells visited (S_chunk) */
    uint64_t chunksEntered;   /* loaded chunks stepped into (E_chunk) */
    uint64_t innerSteps;      /* voxel cells visited */
    uint64_t hits;            /* voxels decompressed (H) */
    uint64_t litVoxels;       /* voxels whose lighting was computed */
    uint64_t degenerate;      /* segments ended at once by D16 (a zero or NaN direction component) */
} dno_counters;

/* Sync: restatement of DN_sync_gpu's per-tile loop (voxel.c:719-786) with the
 * state machine of _DN_stream_to_gpu (voxel.c:1491-1536) and the request rule
 * of _DN_request_chunk_lighting (voxel.c:1463-1489).  The CPU map and chunks
 * are read (not modified; the caller clears 'updated' afterwards as the
 * product does). op: 0 DN_READ, 1 DN_WRITE, 2 DN_READ_WRITE. */
void dno_sync(dno_map* m, const dno_handle* cpuMap, const dno_chunk* chunks,
              const dno_material* materials, int op, int lightingSplit);

/* LRU residency: the reference's GPU voxel buffer of power-of-two nodes (voxel.c:1538-1695), as the
 * product's DN_RESIDENCY_LRU.  dno_set_lru starts it with DN_create_volume's buffer for numChunks chunk
 * slots (before the first sync); dno_set_chunk_cap gives the CPU chunk capacity that bounds the buffer's
 * growth (call it before each sync); dno_lru_nodes exports the nodes in buffer order. */
void dno_set_lru(dno_map* m, uint64_t numChunks);
void dno_set_chunk_cap(dno_map* m, uint64_t chunkCap);
size_t dno_lru_nodes(const dno_map* m, uint64_t* voxelCap, uint32_t* sizes, uint64_t* starts, int64_t* tiles, size_t cap);
/* the node model's steps on their own (a differential test drives them with random sequences):
 * _DN_stream_voxels' choice (1 with a node, *victim the previous owner or -1; 0 without), _DN_unload_voxels,
 * the sort pass, whole-node growth; lastUsed replaced for every tile */
int dno_lru_stream(dno_map* m, int64_t tile, uint32_t nvox, int64_t* victim);
void dno_lru_unload(dno_map* m, int64_t tile);
void dno_lru_sort(dno_map* m, int maxCopies);
void dno_lru_grow(dno_map* m, uint64_t num);
void dno_set_last_used(dno_map* m, const uint32_t* lastUsed);

/* Lighting update over the current request list (voxelLighting.comp:207-288). */
void dno_light(dno_map* m, const dno_material* materials, const dno_light_params* p, int nthreads);

/* Draw (voxelDraw.comp:63-147).  color: RGBA floats per pixel (rgb, depth);
 * hit: global voxel index; face: D14.  With a pixel subset, outputs are
 * packed in subset order. */
void dno_draw(dno_map* m, const dno_material* materials, const dno_draw_params* p,
              float* color, uint32_t* hit, uint8_t* face, int nthreads);

/* Lighting of a subset of requests only (size-independent sampled parity):
 * computes results for the listed request indices without committing.
 * out_diff/out_spec: 32*3 floats per listed request; valid: 32 bytes each. */
void dno_light_requests(dno_map* m, const dno_material* materials, const dno_light_params* p,
                        const uint32_t* reqIdx, uint32_t n, float* out_diff, float* out_spec,
                        uint8_t* valid, int nthreads);

/* --- state access for tests --- */
uint32_t dno_num_requests(const dno_map* m);
const uint32_t* dno_requests(const dno_map* m);     /* (tile << 4) | group, tile order */
uint32_t dno_frame_num(const dno_map* m);
void dno_get_counters(const dno_map* m, dno_counters* out);
void dno_reset_counters(dno_map* m);
/* tile state export: state (0 absent, 1 unloaded, 2 loaded, 3 requested), vis, lastUsed */
void dno_export_tiles(const dno_map* m, uint8_t* state, uint8_t* vis, uint32_t* lastUsed);
/* lighting export for every loaded chunk: rows (globalVoxelIndex, diff rgb, spec rgb) in
 * tile order then rank order; returns the number of rows (call with NULL to count). */
uint64_t dno_export_lighting(const dno_map* m, uint32_t* index, float* diff, float* spec);
/* per-tile sample counts (0 for tiles that are not loaded) */
void dno_export_samples(const dno_map* m, uint32_t* samples);
/* import lighting + samples + vis for loaded chunks from another implementation
 * (rows as in dno_export_lighting); used by sampled parity at full size. */
void dno_import_lighting(dno_map* m, uint64_t n, const uint32_t* index, const float* diff, const float* spec);
void dno_import_samples(dno_map* m, const uint32_t* samples);

/* adopt another implementation's tile states (0..3) and visible flags; loaded tiles are packed
 * from the CPU chunks by this oracle's own packing.  Used to time / check a sample of one frame of
 * a large workload without replaying every earlier frame. */
void dno_import_state(dno_map* m, const dno_handle* cpuMap, const dno_chunk* chunks, const dno_material* materials,
                      const uint8_t* state, const uint8_t* vis, uint32_t frameNum);
void dno_set_requests(dno_map* m, const uint32_t* words, uint32_t n);

/* deterministic sine used by RNG mode A (Cody-Waite reduction + Taylor polynomial) */
float dno_sin(float x);
/* RNG mode B hash */
uint32_t dno_hash32(uint32_t x);
/* K-point golden-angle sphere, computed in double and rounded to float */
void dno_sphere_points(uint32_t K, float out[][3]);

/* Shapes (dno_shapes.c): the reference's shape functions (voxelShapes.c:23-442) on a dense map.  The
 * caller gives each shape's transform and inverse; every kind takes its centre (base for the cone and
 * the pyramid) in c and, by kind: sphere a = r; box v = len; rounded box v = len, a = r; torus a = ra,
 * b = rb; ellipsoid v = radii; cylinder a = r, b = h; cone a = r, b = h; pyramid v = len. */
enum { DNO_SHAPE_SPHERE = 0, DNO_SHAPE_BOX, DNO_SHAPE_ROUNDED_BOX, DNO_SHAPE_TORUS, DNO_SHAPE_ELLIPSOID,
       DNO_SHAPE_CYLINDER, DNO_SHAPE_CONE, DNO_SHAPE_PYRAMID };
typedef struct dno_shape_op {
    int32_t kind, flip;
    uint8_t material, albedo[3];      /* the placed voxel (255 = empty: a removal) */
    float normal[3];                  /* its own normal, kept by removals */
    float c[3], v[3];
    float a, b;
    float transform[4][4], invTransform[4][4];
} dno_shape_op;
typedef struct dno_shape_hit { uint16_t local; uint8_t inside, pad; float normal[3]; } dno_shape_hit;
/* the shape's bounding box after its transform (the sphere's is not transformed) */
void dno_shape_bounds(const dno_shape_op* op, float mn[3], float mx[3]);
/* the covered chunk range inside the map; 0 when empty */
int dno_shape_range(const dno_shape_op* op, const uint32_t mapSize[3], int32_t cmin[3], int32_t cmax[3]);
/* per-chunk hit counts and the hits (up to capacity) in chunk then voxel order; returns the total */
uint64_t dno_shape_eval(const dno_shape_op* op, const int32_t cmin[3], const int32_t cmax[3], uint32_t* counts,
                        dno_shape_hit* hits, uint64_t capacity);
/* applies the hits to a dense map: normal / albedo words per voxel (x + 8X*(y + 8Y*z)), voxel count per tile */
void dno_shape_apply(const dno_shape_op* op, const uint32_t mapSize[3], const int32_t cmin[3], const int32_t cmax[3],
                     const uint32_t* counts, const dno_shape_hit* hits, uint32_t* normalWords, uint32_t* albedoWords,
                     int32_t* tileCount);

#ifdef __cplusplus
}
#endif
#endif
