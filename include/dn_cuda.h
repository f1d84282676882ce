/*
 * dn_cuda.h -- the C ABI between the DN_* host layer and the CUDA kernels
 * (libdoonengine.so).  Plain C types, pointers and sizes only; every entry
 * returns an int status (DN_CUDA_OK = 0) and no exception crosses it.
 *
 * In the reference these operations are OpenGL calls made from
 * src/DoonEngine/voxel.c; each entry below names the call sites it replaces.
 * The device state of one map is an opaque struct DNgpuVolume.
 */
#ifndef DN_CUDA_H
#define DN_CUDA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

struct DNgpuVolume;

enum {
    DN_CUDA_OK = 0,
    DN_CUDA_ERR_ARG = 1,        /* bad argument (size, NULL, out of range) */
    DN_CUDA_ERR_NOMEM = 2,      /* device or pinned allocation failed */
    DN_CUDA_ERR_LAUNCH = 3,     /* kernel launch / CUDA runtime error */
    DN_CUDA_ERR_DEVICE = 4,     /* no usable GPU */
    DN_CUDA_ERR_KERNEL = 5,     /* a kernel flagged an error status */
    DN_CUDA_ERR_CAPACITY = 6    /* fixed-size scratch too small for the request */
};

#define DN_SLOT_NONE 0x3FFFFFFFu

/* material as uploaded with every draw / lighting launch (voxel.h:82-94, 32 B) */
typedef struct dn_material {
    float padding[2];
    uint32_t emissive;
    float opacity, refractIndex, specular;
    uint32_t reflectType, shininess;
} dn_material;

/* one packed chunk (the packing of voxel.c:1397-1461): the input of dn_cuda_sync; dn_cuda_sync_chunks reads
 * only pos, nvox and voxBase and packs the rest on the device */
typedef struct dn_chunk_record {
    uint32_t mask[16];      /* bit x + 8*(y + 8*z) */
    uint32_t partial[3];    /* set bits before 128, 256, 384 */
    uint32_t nvox;          /* set bits */
    int32_t pos[3];         /* chunk position in the map */
    uint32_t voxBase;       /* first voxel in the device pool */
} dn_chunk_record;

/* per-tile pending operation decided by the host at sync (voxel.c:1491-1536) */
#define DN_PEND_VALID   0x1u   /* the entry carries CPU-side state for the tile */
#define DN_PEND_EXISTS  0x2u   /* the chunk exists on the CPU (DNchunkHandle.flag != 0) */
#define DN_PEND_UPDATED 0x4u   /* DNchunk.updated was set */
#define DN_PEND_STAGED  0x8u   /* a freshly packed record was staged into 'slot' */
/* DN_RESIDENCY_LRU decisions of the host's node model (voxel.c:1554-1630); the tile's record slot is
 * dropped with an eviction */
#define DN_PEND_EVICT   0x10u  /* a later tile of this sync took the chunk's node: unloaded after its requests */
#define DN_PEND_EVICTED 0x20u  /* an earlier tile of this sync took the chunk's node: unloaded before its turn */
#define DN_PEND_HOLD    0x40u  /* the requested chunk found no node: unloaded again, lastUsed 0 */
typedef struct dn_tile_op {
    uint32_t tile;
    uint32_t flags;
    uint32_t slot;          /* record slot of the staged chunk (DN_PEND_STAGED) */
    uint32_t recordIndex;   /* index into the records array of the same call */
} dn_tile_op;

typedef struct dn_sync_params {
    uint32_t op;            /* 0 DN_READ, 1 DN_WRITE, 2 DN_READ_WRITE */
    uint32_t split;         /* lightingSplit >= 1 */
    uint32_t frameNum;
} dn_sync_params;

typedef struct dn_light_params {
    float sunDir[3];        /* normalised (voxel.c:942) */
    float sunStrength[3], ambient[3], camPos[3], skyBot[3], skyTop[3];
    float shadowSoftness, time, emissiveStrength;
    uint32_t numDiffuse, maxDiffuse, diffuseBounceLimit, specBounceLimit;
    uint32_t K;             /* direct / specular rays, 1..64 */
    uint32_t rngMode;       /* 0 hash, 1 sin-fract */
    uint32_t mapId;
    float spherePts[64][3];
} dn_light_params;

typedef struct dn_draw_params {
    float origin[3];        /* invView * (0,0,0,1) */
    float dirMat[4][4];     /* invCenteredView * invProjection, column-major */
    uint32_t width, height, viewMode, truncate16;
    float sunStrength[3], skyBot[3], skyTop[3];
    float emissiveStrength;
    /* raster composition (voxelDraw.comp:86-101, 127-136), used when compose is 1: device textures of the
     * rasterised scene, texel (i, j) at [j * w + i] like the output's pixels; colour RGBA32F (alpha unused),
     * depth one float per texel (window depth, 0 near .. 1 far) */
    float invProj[4][4];        /* inverse projection, column-major */
    const float* rasterColor;
    const float* rasterDepth;
    uint32_t rasterColorW, rasterColorH, rasterDepthW, rasterDepthH;
    uint32_t compose;
} dn_draw_params;

typedef struct dn_stats {
    uint64_t rays, primary, outerSteps, chunksEntered, innerSteps, hits, litVoxels;
    uint64_t degenerate;    /* segments ended at once for a zero or NaN direction component */
} dn_stats;

/* --- device lifetime: replaces DN_init's buffer / program setup (voxel.c:119-154) and DN_quit (156-163) --- */
int dn_cuda_init(int device);
void dn_cuda_shutdown(void);
const char* dn_cuda_error_string(int code);
/* last detailed error message of this thread */
const char* dn_cuda_last_error(void);

/* --- map lifetime: replaces the SSBO creation of DN_create_volume (voxel.c:173-195) and glDeleteBuffers (285-287) --- */
int dn_cuda_map_create(uint32_t sx, uint32_t sy, uint32_t sz, uint32_t slotCap, uint64_t voxelCap,
                       struct DNgpuVolume** out);
void dn_cuda_map_destroy(struct DNgpuVolume* g);
/* re-creates the tile arrays for a new map size, every tile absent (DN_set_map_size, voxel.c:989-1007) */
int dn_cuda_map_resize(struct DNgpuVolume* g, uint32_t sx, uint32_t sy, uint32_t sz);
/* grows the record slots / voxel pool / request capacity, keeping contents
 * (DN_set_max_voxels_gpu voxel.c:1042-1061; request buffer voxel.c:898-916) */
int dn_cuda_reserve(struct DNgpuVolume* g, uint32_t slotCap, uint64_t voxelCap, uint64_t requestCap);

/* --- sync: replaces glMapBuffer of the map buffer and the per-tile host loop of DN_sync_gpu
 *     (voxel.c:729-770), the request build (1463-1489), the chunk / voxel uploads
 *     (1548-1552, 1636-1637) and the request upload of DN_update_lighting (919).
 *     ops: pending per-tile CPU-side state; records: packed chunks for the staged ops;
 *     voxels: 2 words per voxel, record r's voxels at voxels[2*records[r].voxBase ...] are
 *     taken from 'voxelWords' in record order (concatenated). --- */
int dn_cuda_sync(struct DNgpuVolume* g, const dn_sync_params* p,
                 const dn_tile_op* ops, uint32_t nops,
                 const dn_chunk_record* records, uint32_t nrecords,
                 const uint32_t* voxelWords, uint64_t nvoxels);

/* --- lighting: replaces glDispatchCompute(numLightingRequests) of DN_update_lighting (voxel.c:950) --- */
int dn_cuda_light(struct DNgpuVolume* g, const dn_light_params* p, const dn_material* materials);

/* Lighting update that allocates nothing (no counterpart in the reference, which has no such
 * constraint).  For callers that must not allocate device memory while a frame is in flight -- a render
 * loop under a fixed device-memory budget, or a host engine whose own allocator owns all device memory --
 * the per-request scratch that dn_cuda_light keeps in the volume (grown with cudaMalloc by dn_cuda_sync)
 * is replaced by a fixed 8 MiB array in the library's device image, held by every GPU that loads the
 * library until the process exits.  Same inputs, outputs and kernels as dn_cuda_light.
 * Limit: 8192 request groups (262144 voxels) per call, or the lower limit set below.  The request count
 * is known only on the device, so the check runs there and the call never waits for the GPU: a list
 * above the limit is not lit at all (the volume is left unchanged) and the next dn_cuda_finish (DN_finish)
 * returns DN_CUDA_ERR_CAPACITY with a message naming the limit.
 * The first call on a device looks up the array's device address (with that device current); make that
 * first call before any stream capture.  dn_cuda_init and dn_cuda_shutdown drop the looked-up addresses,
 * so after a device reset call dn_cuda_init again before the next call.  Calls share the array: calls
 * that overlap on the GPU race. */
int dn_cuda_light_noalloc(struct DNgpuVolume* g, const dn_light_params* p, const dn_material* materials);
/* Lowers the per-call limit of dn_cuda_light_noalloc to 'groups' request groups (0 or more than 8192:
 * back to 8192); returns the previous limit.  Process-wide. */
uint32_t dn_cuda_light_noalloc_set_limit(uint32_t groups);

/* --- draw: replaces glDispatchCompute(w/16, h/16) of DN_draw (voxel.c:879); outputs are device pointers --- */
int dn_cuda_draw(struct DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials,
                 float* colorOut, uint32_t* hitOut, uint8_t* faceOut);
/* draw into host memory: device staging plus asynchronous copies; valid after dn_cuda_finish */
int dn_cuda_draw_host(struct DNgpuVolume* g, const dn_draw_params* p, const dn_material* materials,
                      float* colorOut, uint32_t* hitOut, uint8_t* faceOut);

/* The staging half of dn_cuda_sync: uploads and publishes the ops, records and voxels without the
 * per-tile pass (for maps whose per-tile pass runs in a batched frame, DN_BATCH_SYNC). */
int dn_cuda_sync_stage(struct DNgpuVolume* g, const dn_tile_op* ops, uint32_t nops,
                       const dn_chunk_record* records, uint32_t nrecords,
                       const uint32_t* voxelWords, uint64_t nvoxels);

/* --- sync with packing on the device (no counterpart in the reference, which packs on the host,
 *     voxel.c:1397-1461).  Each staged record comes with its chunk's 512 voxels as the CPU map stores them
 *     (DNcompressedVoxel voxels[8][8][8]: normal word, sRGB albedo word; x outermost).  The device does the
 *     packing: the surface cull (a solid voxel is kept when a face neighbour is outside the chunk, empty or
 *     of a see-through material), the occupancy mask and partial counts, the compaction in mask order and
 *     the albedo linearisation.  The host supplies, per record, pos, voxBase and nvox: the kept-voxel
 *     count, which sizes the record's pool range before the upload; the device counts again and a record
 *     whose count differs is not published (its tile stays unloaded; dn_cuda_finish reports
 *     DN_CUDA_ERR_KERNEL).  mask and partial of the records are not read. --- */
typedef struct dn_pack_params {
    uint32_t seeThrough[8];  /* bit m: material m is empty (255) or has opacity < 1 */
    uint8_t linear[256];     /* sRGB albedo byte -> linear byte (voxel.c:1441-1447) */
} dn_pack_params;
/* chunkVoxels[r]: the 4096-byte voxel array of record r; copied before the call returns.  A sync whose
 * chunks exceed the volume's staging buffer (16 MiB) is uploaded in parts, and the call then waits for
 * each part's upload before it fills the buffer again. */
int dn_cuda_sync_chunks(struct DNgpuVolume* g, const dn_sync_params* p, const dn_pack_params* pk,
                        const dn_tile_op* ops, uint32_t nops,
                        const dn_chunk_record* records, uint32_t nrecords, const void* const* chunkVoxels);
/* Sets the size of one staging part of dn_cuda_sync_chunks (0: back to 16 MiB); returns the previous size.
 * Process-wide; for tests of the multi-part upload. */
size_t dn_cuda_stage_part_limit(size_t bytes);
/* the staging half of dn_cuda_sync_chunks (DN_BATCH_SYNC maps; see dn_cuda_sync_stage) */
int dn_cuda_sync_stage_chunks(struct DNgpuVolume* g, const dn_pack_params* pk,
                              const dn_tile_op* ops, uint32_t nops,
                              const dn_chunk_record* records, uint32_t nrecords, const void* const* chunkVoxels);
/* the device record of a loaded tile and its voxel words (2 per voxel: normal, linear albedo; room for 512
 * voxels); waits for the map's stream.  Returns DN_CUDA_ERR_ARG when the tile has no record. */
int dn_cuda_export_chunk(struct DNgpuVolume* g, uint32_t tile, dn_chunk_record* rec, uint32_t matSet[8],
                         uint32_t* words);

/* --- batches (no counterpart in the reference, which issues one GL dispatch sequence per volume) ---
 * A batch runs the frame work of many maps as kernels that each cover every map of the frame: one draw
 * launch over all maps' pixels, one launch of the per-tile sync pass over all maps' tiles, one persistent
 * lighting launch over a device-side queue of every map's lighting requests, one commit launch.  Each map's
 * results are exactly those of the single-map calls (dn_cuda_draw, dn_cuda_sync, dn_cuda_light) with the
 * same arguments.  Member volumes run all their work on the batch's stream.  A frame whose composition
 * repeats (same maps, phases, images and device arrays) is replayed as one CUDA graph. */
struct DNgpuBatch;

#define DN_BATCH_DRAW  0x1u   /* dn_cuda_draw / dn_cuda_draw_host with 'draw' */
#define DN_BATCH_SYNC  0x2u   /* the per-tile pass of dn_cuda_sync with 'sync' (ops staged before) */
#define DN_BATCH_LIGHT 0x4u   /* dn_cuda_light with 'light' */

typedef struct dn_batch_item {
    struct DNgpuVolume* map;
    uint32_t phases;            /* DN_BATCH_*; phases run in the order draw, sync, light */
    uint32_t hostImage;         /* 1: colorOut / hitOut / faceOut are host memory (valid after finish) */
    const dn_material* materials;   /* 256 entries */
    dn_draw_params draw;
    float* colorOut;            /* width * height * 4 floats */
    uint32_t* hitOut;           /* optional */
    uint8_t* faceOut;           /* optional */
    dn_sync_params sync;
    dn_light_params light;
} dn_batch_item;

/* knobs of the batched lighting launch, chosen by dn_cuda_batch_autotune */
typedef struct dn_batch_tuning {
    uint32_t streamBatch;       /* compaction period of the ray pools: lanes of a warp whose segment ended
                                   before the warp regroups (shades them and refills them from the pool), 1..32 */
    uint32_t blocksPerSM;       /* resident lighting blocks per SM */
    uint32_t useGraph;          /* replay repeated frames as a CUDA graph */
    uint32_t kernel;            /* lighting kernel: 1 per-lane ray streams, 2 warp packets of ray fans */
    uint32_t poolRays;          /* rays per warp: rays of each fan kind a warp pulls into one pool, 64 or 128 */
    uint32_t diffuseBatch;      /* the diffuse-path kernel's compaction period (lanes waiting before refill) */
} dn_batch_tuning;

int dn_cuda_batch_create(struct DNgpuBatch** out);
/* removes every member (their work returns to their own streams) and frees the batch */
void dn_cuda_batch_destroy(struct DNgpuBatch* b);
int dn_cuda_batch_add(struct DNgpuBatch* b, struct DNgpuVolume* g);
int dn_cuda_batch_remove(struct DNgpuBatch* b, struct DNgpuVolume* g);
/* one frame: every item's phases; each map at most once; every map a member of b */
int dn_cuda_batch_frame(struct DNgpuBatch* b, const dn_batch_item* items, uint32_t n);
/* waits for the batch's work; reports kernel error flags of every member */
int dn_cuda_batch_finish(struct DNgpuBatch* b);
/* counters of batched launches (kind 0 all, 1 draw, 2 lighting); single-map calls count on their map */
int dn_cuda_batch_stats(struct DNgpuBatch* b, int kind, dn_stats* out);
int dn_cuda_batch_reset_stats(struct DNgpuBatch* b);
void* dn_cuda_batch_stream(struct DNgpuBatch* b);
int dn_cuda_batch_get_tuning(struct DNgpuBatch* b, dn_batch_tuning* out);
int dn_cuda_batch_set_tuning(struct DNgpuBatch* b, const dn_batch_tuning* t);
/* Times the lighting launch of the last batched frame under each candidate tuning, keeps the fastest and
 * returns it in chosen (may be NULL).  Every map's state is left as it was: the reruns write only scratch,
 * and the requested / touched / visible flags they set are saved before and restored after.  Call after a
 * frame with DN_BATCH_LIGHT items. */
int dn_cuda_batch_autotune(struct DNgpuBatch* b, dn_batch_tuning* chosen);
/* request groups of the map's last sync, as read by its last dn_cuda_finish or dn_cuda_batch_finish */
uint64_t dn_cuda_requests_of(struct DNgpuVolume* g);

/* --- residency (no counterpart in the reference; used by the serving loop's admission control) ---
 * A map's device bytes (persistent arrays plus scratch).  Eviction waits for the map's work, copies its
 * persistent state (tiles, records, voxel pool and FP32 lighting, request list, status) to pinned host
 * memory and frees all its device memory; restore brings it back, after which the map behaves exactly as
 * if it had never left.  Other entries reject an evicted map with DN_CUDA_ERR_ARG. */
uint64_t dn_cuda_map_footprint(struct DNgpuVolume* g);
int dn_cuda_map_is_resident(struct DNgpuVolume* g);
int dn_cuda_map_evict(struct DNgpuVolume* g);
int dn_cuda_map_restore(struct DNgpuVolume* g);
/* Restore without making the volume's stream wait: the allocations and copies are queued on the restore
 * stream and the call returns at once.  dn_cuda_map_restore_query returns 1 once the copies are done (and
 * for a resident volume with nothing pending), 0 while they run or the volume is evicted, -1 on error.  A
 * server admits the volume to its next tick only then, so its other volumes' work never waits for the
 * copies.  Any other entry point (dn_cuda_map_restore included) used on the volume first makes its stream
 * wait for them. */
int dn_cuda_map_restore_async(struct DNgpuVolume* g);
int dn_cuda_map_restore_query(struct DNgpuVolume* g);
/* Evictions copy into a process-wide pool of pinned 64 MiB host slabs, pinned when first needed and reused
 * by every volume afterwards.  dn_cuda_host_reserve pins slabs until the pool holds 'bytes', so that no
 * eviction under load has to pin host memory (a server whose volumes exceed its device budget reserves the
 * difference at start); dn_cuda_host_pinned returns the pool's size in bytes. */
int dn_cuda_host_reserve(uint64_t bytes);
uint64_t dn_cuda_host_pinned(void);
/* the pool's free bytes (slabs no evicted volume holds), and pinning until at least 'bytes' are free (a
 * server pins ahead while idle: evictions of smaller maps take more slabs for the same bytes) */
uint64_t dn_cuda_host_pinned_free(void);
int dn_cuda_host_headroom(uint64_t bytes);
/* the size of one slab of the pool (64 MiB) */
uint64_t dn_cuda_host_slab_bytes(void);
/* 1 when the work recorded by ev has completed, 0 while pending, negative on error */
int dn_cuda_event_query(void* ev);

/* --- synchronisation, counters, introspection (additions) --- */
int dn_cuda_finish(struct DNgpuVolume* g, uint64_t* numRequests);
int dn_cuda_stats(struct DNgpuVolume* g, dn_stats* out);
/* kind 0: all kernels, 1: draw, 2: lighting */
int dn_cuda_stats_kind(struct DNgpuVolume* g, int kind, dn_stats* out);
int dn_cuda_reset_stats(struct DNgpuVolume* g);
void* dn_cuda_stream(struct DNgpuVolume* g);
int dn_cuda_export_tiles(struct DNgpuVolume* g, uint8_t* state, uint8_t* vis, uint32_t* lastUsed, uint32_t* samples);
/* the per-tile requested and touched bytes the rays set since the last sync (waits for the map's stream);
 * the host's residency model reads them before it decides a sync */
int dn_cuda_read_tile_flags(struct DNgpuVolume* g, uint8_t* requested, uint8_t* touched);
int dn_cuda_export_requests(struct DNgpuVolume* g, uint32_t* out, uint64_t capacity, uint64_t* count);
/* lighting of every loaded chunk; rows ordered by tile then rank */
int dn_cuda_export_lighting(struct DNgpuVolume* g, uint32_t* index, float* diff, float* spec,
                            uint64_t capacity, uint64_t* count);

/* --- shapes: the per-voxel signed-distance pass of the shape functions (voxelShapes.c:150-441) over the
 *     chunk range a shape covers, on the device.  The host applies the resulting edits to the CPU map in
 *     the reference's order (voxelShapes.c:183-232), so the map's contents are the reference's. --- */
enum {
    DN_SHAPE_SPHERE = 0, DN_SHAPE_BOX = 1, DN_SHAPE_ROUNDED_BOX = 2, DN_SHAPE_TORUS = 3,
    DN_SHAPE_ELLIPSOID = 4, DN_SHAPE_CYLINDER = 5, DN_SHAPE_CONE = 6, DN_SHAPE_PYRAMID = 7
};
typedef struct dn_shape_params {
    uint32_t kind;              /* DN_SHAPE_* */
    uint32_t removing;          /* the placed voxel is empty: inside voxels need no normal */
    uint32_t flipNormals;       /* with removing: also report the shell (distance in [0, 1)) */
    float invTransform[4][4];   /* voxel coordinates -> shape space, column-major */
    float center[3];            /* sphere centre */
    float r2, r12;              /* sphere: r*r and (r+1)*(r+1) */
    float radius, radiusB, height;
    float angles[2];            /* cone: (h, r) / sqrt(r*r + h*h) */
    float radii[3];             /* ellipsoid semi-axes */
    float length[3];            /* box / rounded box half extents; pyramid base (x, z) */
    int32_t chunkMin[3], chunkMax[3];   /* inclusive chunk range, inside the map */
} dn_shape_params;

/* a voxel the shape touches: local = x + 8*(y + 8*z) within its chunk; inside 1 (distance < 0) or 0 (a
 * shell voxel of a removal with flipped normals); normal as the reference computes it before flipping
 * (zero for inside voxels of a removal) */
typedef struct dn_shape_hit {
    uint16_t local;
    uint8_t inside;
    uint8_t pad;
    float normal[3];
} dn_shape_hit;

/* Evaluates p over every voxel of its chunk range on the current device (synchronous).  counts (host,
 * one per chunk of the range, chunk i = x + nx*(y + ny*z) relative to chunkMin) receives each chunk's hit
 * count; *hits the hits of all chunks in chunk order, each chunk's in voxel order z, y, x; *total their
 * number.  *hits stays valid until dn_cuda_shape_free(*hits), to be called once per successful call
 * (the calling thread's buffers, reused by its next call). */
int dn_cuda_shape_eval(const dn_shape_params* p, uint32_t* counts, dn_shape_hit** hits, uint64_t* total);
void dn_cuda_shape_free(dn_shape_hit* hits);
/* voxels evaluated and device time of the evaluation kernels (both passes) since the last reset */
void dn_cuda_shape_stats(uint64_t* voxels, double* deviceMs, int reset);

/* device / pinned memory and event helpers for callers without their own CUDA runtime */
int dn_cuda_malloc(void** p, size_t bytes);
int dn_cuda_free(void* p);
int dn_cuda_malloc_host(void** p, size_t bytes);
int dn_cuda_free_host(void* p);
int dn_cuda_memcpy_d2h(void* dst, const void* src, size_t bytes);
/* complete when it returns: later work on any of the library's streams sees the bytes */
int dn_cuda_memcpy_h2d(void* dst, const void* src, size_t bytes);
int dn_cuda_event_create(void** ev);
int dn_cuda_event_destroy(void* ev);
int dn_cuda_event_record(void* ev, void* stream);
int dn_cuda_event_elapsed_ms(void* start, void* end, float* ms);
int dn_cuda_stream_sync(void* stream);
int dn_cuda_device_sync(void);
/* writes 'bytes' of a scratch buffer on 'stream' (L2 flush between timed steps) */
int dn_cuda_flush_l2(void* stream, size_t bytes);
/* number of kernels this library has launched since load (all volumes) */
uint64_t dn_cuda_launch_count(void);
/* number of device and pinned-host allocations this library has made since load (all threads) */
uint64_t dn_cuda_alloc_count(void);
/* names of the kernels this library launches, ';'-separated */
const char* dn_cuda_kernel_names(void);

#ifdef __cplusplus
}
#endif
#endif
