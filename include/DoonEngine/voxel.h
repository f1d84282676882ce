/*
 * voxel.h -- the DoonEngine DN_* C API, GL-free, backed by CUDA kernels for
 * sm_103a (GB300).
 *
 * Drop-in for the reference's src/DoonEngine/voxel.h (lines cited per item):
 * same function names, argument meaning, 8x8x8-chunk map layout and error
 * behaviour (bool / NULL / -1 returns plus g_DN_message_callback).  OpenGL
 * objects are replaced as follows:
 *   - the three GL buffer IDs of DNvolume (voxel.h:100-102) become one opaque
 *     device handle, `gpu`;
 *   - DN_draw's GL_RGBA32F output texture (voxel.h:207) becomes a DNimage
 *     (RGBA32F colour + depth, plus the hit voxel index and face per pixel),
 *     in device or host memory;
 *   - the raster colour / depth texture handles stay as ints; -1 means "no
 *     raster composition" exactly as in the reference.  The textures are
 *     device buffers made with DN_texture_create (addition) in place of the
 *     GL textures of the application's raster pass;
 *   - the cube-map sky (voxel.h:135-136) is not available (no texture stack);
 *     the gradient sky is used and useCubemap is ignored with a NOTE.
 * Additions are marked "addition".
 */
#ifndef DN_VOXEL_H
#define DN_VOXEL_H

#ifdef __cplusplus
extern "C"
{
#endif

#include "globals.h"
#include "dn_math.h"
#include <stdbool.h>
#include <stdint.h>

/* voxel.h:17-31 */
#define DN_CHUNK_SIZE 8
#define DN_CHUNK_LENGTH 512
#define DN_MAX_MATERIALS 256
#define DN_MATERIAL_EMPTY 255
#define DN_GAMMA 2.2f
#define DN_FLATTEN_INDEX(p, s) (p.x) + (s.x) * ((p.y) + (p.z) * (s.y))

/* voxel.h:35-46 */
typedef struct DNcolor { uint8_t r, g, b; } DNcolor;

typedef struct DNvoxel
{
	uint8_t material; /* [0, 255]; 255 = empty */
	DNvec3 normal;
	DNcolor albedo;
} DNvoxel;

/* voxel.h:49-53: normal = material<<24 | n.x<<16 | n.y<<8 | n.z ; albedo = r<<24 | g<<16 | b<<8 */
typedef struct DNcompressedVoxel
{
	uint32_t normal;
	uint32_t albedo;
} DNcompressedVoxel;

/* voxel.h:56-64 (same layout; voxels indexed [x][y][z]) */
typedef struct DNchunk
{
	DNivec3 pos;
	bool updated;
	uint32_t numVoxels;
	uint32_t numVoxelsGpu;
	DNcompressedVoxel voxels[8][8][8];
} DNchunk;

/* voxel.h:67-71 */
typedef struct DNchunkHandle
{
	uint8_t flag;        /* 0 = does not exist, 1 = exists on the CPU */
	uint32_t chunkIndex;
} DNchunkHandle;

/* voxel.h:74-79.  Kept for source compatibility; the device pool allocator
 * does not expose a node list (gpuVoxelLayout is NULL). */
typedef struct DNvoxelNode
{
	uint32_t size;
	size_t startPos;
	DNivec3 chunkPos;
} DNvoxelNode;

/* voxel.h:82-94 (32 bytes, the std140 layout the reference uploads) */
typedef struct DNmaterial
{
	DNvec2 padding;
	uint32_t emissive;
	float opacity;
	float refractIndex;
	float specular;
	uint32_t reflectType;  /* 0: no sky reflection, 1: reflect sky colour, 2: highlight only */
	uint32_t shininess;
} DNmaterial;

struct DNgpuVolume;   /* opaque device-side map (dn_cuda.h) */

/* voxel.h:97-142.  Field meaning and READ ONLY / READ-WRITE contracts as in
 * the reference. */
typedef struct DNvolume
{
	struct DNgpuVolume* gpu;         /* READ ONLY  | device-side map (replaces the three GL buffer IDs) */

	DNuvec3 mapSize;                 /* READ ONLY  | size of the map in chunks */
	size_t chunkCap;                 /* READ ONLY  | CPU chunk capacity */
	size_t nextChunk;                /* READ ONLY  | next probably-free chunk index */
	size_t voxelCap;                 /* READ ONLY  | device voxel pool capacity, in voxels */
	size_t numVoxelNodes;            /* READ ONLY  | number of chunks staged in the device pool */
	size_t numLightingRequests;      /* READ ONLY  | request words built by the last DN_sync_gpu (filled in by DN_finish) */
	size_t lightingRequestCap;       /* READ ONLY  | device request capacity */

	DNchunkHandle* map;              /* READ-WRITE | mapSize.x*y*z handles */
	DNchunk* chunks;                 /* READ-WRITE | chunkCap chunks */
	DNmaterial* materials;           /* READ-WRITE | 256 materials */
	uint32_t* lightingRequests;      /* READ-WRITE | NULL: requests are built and kept on the device */
	DNvoxelNode* gpuVoxelLayout;     /* READ ONLY  | NULL (see DNvoxelNode) */

	DNvec3 camPos;                   /* READ-WRITE | camera position, in chunks */
	DNvec3 camOrient;                /* READ-WRITE | {pitch, yaw, roll} in degrees */
	float camFOV;                    /* READ-WRITE | degrees */
	uint32_t camViewMode;            /* READ-WRITE | 0 lighting, 1 albedo, 2 diffuse, 3 specular, 4 voxel normals, 5 face normals */

	DNvec3 sunDir;                   /* READ-WRITE */
	DNvec3 sunStrength;              /* READ-WRITE */
	DNvec3 ambientLightStrength;     /* READ-WRITE */
	uint32_t diffuseBounceLimit;     /* READ-WRITE */
	uint32_t specBounceLimit;        /* READ-WRITE */
	float shadowSoftness;            /* READ-WRITE */

	bool useCubemap;                 /* READ-WRITE | ignored: cube-map sky is unavailable (no texture stack) */
	uint32_t glCubemapTex;           /* READ-WRITE | ignored */
	DNvec3 skyGradientBot;           /* READ-WRITE */
	DNvec3 skyGradientTop;           /* READ-WRITE */

	uint32_t frameNum;               /* READ ONLY */
	float lastTime;                  /* READ ONLY */

	/* additions */
	float emissiveStrength;          /* READ-WRITE | scale of emissive voxels (1.0 = reference) */
	uint32_t numDirectRays;          /* READ-WRITE | K fixed direct-light and specular rays per voxel (1..64, default 15) */
	uint32_t rngMode;                /* READ-WRITE | 0 = per-ray integer hash (default), 1 = reference sin-fract */
	uint32_t mapId;                  /* READ-WRITE | random-stream key of this map */
	uint32_t truncateDispatch;       /* READ-WRITE | 1 = skip the right/bottom pixels the reference's w/16 x h/16 dispatch drops */
	uint64_t deviceBudgetBytes;      /* READ-WRITE | reserved (0); the device pool grows instead of evicting chunks; whole-volume eviction under a device budget is the serving layer's (serve.h) */
} DNvolume;

/* voxel.h:145-150 */
typedef enum DNmemOp
{
	DN_READ,
	DN_WRITE,
	DN_READ_WRITE
} DNmemOp;

/* addition: the draw target that replaces the GL texture */
typedef struct DNimage
{
	uint32_t width, height;
	float* color;         /* RGBA32F per pixel: rgb (gamma corrected) and depth, like the reference texture */
	uint32_t* hitIndex;   /* optional: global voxel index x + X*(y + Y*z) of the hit voxel, 0xFFFFFFFF on a miss */
	uint8_t* hitFace;     /* optional: 0 +x, 1 -x, 2 +y, 3 -y, 4 +z, 5 -z, 6 none */
	int onDevice;         /* 1: device pointers; 0: host pointers (copied back asynchronously; valid after DN_finish) */
} DNimage;

/* addition: traversal counters */
typedef struct DNstats
{
	uint64_t rays;            /* traversal segments (step_map calls) of every kind */
	uint64_t primaryRays;
	uint64_t outerSteps;      /* chunk cells visited */
	uint64_t chunksEntered;   /* loaded chunks stepped into */
	uint64_t innerSteps;      /* voxel cells visited */
	uint64_t hits;            /* voxels read */
	uint64_t litVoxels;       /* voxels whose lighting was updated */
	uint64_t degenerate;      /* segments ended at once for a zero or NaN direction component */
} DNstats;

/* INITIALIZATION (voxel.h:153-184) */
bool DN_init(void);
void DN_quit(void);
DNvolume* DN_create_volume(DNuvec3 mapSize, unsigned int minChunks);
void DN_delete_volume(DNvolume* vol);
DNvolume* DN_load_volume(const char* filePath, unsigned int minChunks);
bool DN_save_volume(const char* filePath, DNvolume* vol);

/* DRAWING (voxel.h:186-215) */
void DN_set_view_projection_matrices(DNvolume* vol, float aspectRatio, float nearPlane, float farPlane, DNmat4* view, DNmat4* projection);
void DN_draw(DNvolume* vol, DNimage* output, DNmat4 view, DNmat4 projection, int rasterColorTexture, int rasterDepthTexture);
void DN_update_lighting(DNvolume* vol, int numDiffuseSamples, int maxDiffuseSamples, float time);

/* MEMORY (voxel.h:217-237) */
int DN_add_chunk(DNvolume* vol, DNivec3 pos);
void DN_remove_chunk(DNvolume* vol, DNivec3 pos);
void DN_sync_gpu(DNvolume* vol, DNmemOp op, int lightingSplit);

/* MAP SETTINGS (voxel.h:239-267) */
bool DN_set_map_size(DNvolume* vol, DNuvec3 size);
bool DN_set_max_chunks(DNvolume* vol, size_t num);
bool DN_set_max_voxels_gpu(DNvolume* vol, size_t num);
bool DN_set_max_lighting_requests(DNvolume* vol, size_t num);

/* Device residency of chunks.
 *   DN_RESIDENCY_KEEP (default): a chunk loads at the sync after a ray requests it and stays loaded until
 *     it is edited or removed; the device pool grows as needed.
 *   DN_RESIDENCY_LRU: the reference's fixed GPU voxel buffer (voxel.c:1538-1695): power-of-two nodes of
 *     16..512 voxels in a buffer of 512 * min(tiles, minChunks) / 2 voxels.  A requested chunk takes the
 *     smallest free node that fits, else the node of the loaded chunk unused for the most syncs (more
 *     than one), which is unloaded and must be requested again; with neither, it stays unloaded and the
 *     buffer doubles (up to 512 voxels per chunk slot) at the end of the sync.  Each sync reads the
 *     rays' request and use flags back from the device first, so it waits for the map's earlier work.
 * Set before the volume's first DN_sync_gpu, outside a batch; false otherwise. */
typedef enum DNresidency { DN_RESIDENCY_KEEP = 0, DN_RESIDENCY_LRU = 1 } DNresidency;
bool DN_set_residency(DNvolume* vol, DNresidency mode);
DNresidency DN_get_residency(const DNvolume* vol);
/* DN_RESIDENCY_LRU: the node buffer's size in voxels (*voxelCap) and its nodes in buffer order -- size,
 * first voxel, owning tile or -1 -- for up to 'capacity' nodes (NULL arrays: count only).  Returns the
 * node count (0 with DN_RESIDENCY_KEEP). */
size_t DN_residency_nodes(const DNvolume* vol, size_t* voxelCap, uint32_t* sizes, uint64_t* starts, int64_t* tiles,
                          size_t capacity);

/* MAP UTILITY (voxel.h:269-344) */
bool DN_in_map_bounds(DNvolume* vol, DNivec3 pos);
bool DN_in_chunk_bounds(DNivec3 pos);
DNvoxel DN_get_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos);
DNcompressedVoxel DN_get_compressed_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos);
void DN_set_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos, DNvoxel voxel);
void DN_set_compressed_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos, DNcompressedVoxel voxel);
void DN_remove_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos);
bool DN_does_chunk_exist(DNvolume* vol, DNivec3 pos);
bool DN_does_voxel_exist(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos);
bool DN_step_map(DNvolume* vol, DNvec3 rayDir, DNvec3 rayPos, int maxSteps, DNivec3* hitPos, DNvoxel* hitVoxel, DNivec3* hitNormal);

/* GENERAL UTILITY (voxel.h:346-371) */
void DN_separate_position(DNivec3 pos, DNivec3* mapPos, DNivec3* chunkPos);
DNvec3 DN_cam_dir(DNvec3 orient);
DNcompressedVoxel DN_compress_voxel(DNvoxel voxel);
DNvoxel DN_decompress_voxel(DNcompressedVoxel voxel);

/* ---- additions ---- */

/* Waits for the volume's device work (and host-image copies) to finish and
 * refreshes numLightingRequests.  Returns false if a kernel reported an
 * error (the message callback says which). */
bool DN_finish(DNvolume* vol);

/* Image helpers: device images live in HBM; host images use pinned memory. */
DNimage* DN_image_create(uint32_t width, uint32_t height, int onDevice, int withHitInfo);
void DN_image_destroy(DNimage* img);

/* Raster textures (addition): the colour and depth textures of the reference's raster pass
 * (main.c:310-322) that DN_draw composes with the voxel scene (voxelDraw.comp:86-136), as device
 * buffers.  The handle (> 0) is passed as DN_draw's rasterColorTexture / rasterDepthTexture; composition
 * happens when both name a texture (0 and negative handles name none, as GL never names a created texture
 * 0).  Colour: RGBA32F per texel, alpha unused.  Depth: one float per texel, the window depth (0 at the near
 * plane, 1 at the far plane or where nothing was rasterised).  Texel (i, j) is at [j * width + i], rows in
 * the order of DNimage's pixels.  A draw samples both GL_LINEAR with GL_REPEAT at texture coordinate
 * (x / colourWidth, y / colourHeight), as the reference's textures are set up. */
typedef enum DNtextureFormat
{
	DN_TEXTURE_RGBA32F = 0,
	DN_TEXTURE_DEPTH32F = 1
} DNtextureFormat;
int DN_texture_create(uint32_t width, uint32_t height, DNtextureFormat format);   /* handle, or -1 */
/* waits for device work in flight, then frees the texture */
void DN_texture_destroy(int texture);
/* copies the whole texture from host memory (4 or 1 floats per texel); complete when it returns.  Draws
 * that read the texture must have finished (DN_finish) before it is overwritten. */
bool DN_texture_upload(int texture, const float* texels);
/* the texture's format, or -1 for a handle that names no texture */
int DN_texture_format(int texture);
/* the texture's device buffer, for a CUDA rasteriser that writes it in place (NULL for a bad handle) */
float* DN_texture_device_pointer(int texture, uint32_t* width, uint32_t* height);

/* addition: a dense copy of the CPU map (tools, tests): per voxel x + 8X*(y + 8Y*z) of the whole map the
 * compressed normal word (0xFFFFFFFF where the tile has no chunk) and albedo word (0 for empty voxels);
 * tileFlags (may be NULL) the DNchunkHandle flag of every tile */
void DN_export_voxels(const DNvolume* vol, uint32_t* normalWords, uint32_t* albedoWords, uint8_t* tileFlags);

/* The inverse matrices DN_draw derives from view / projection
 * (voxel.c:845-853): inverse view, inverse view without translation,
 * inverse projection. */
void DN_draw_matrices(DNmat4 view, DNmat4 projection, DNmat4* invView, DNmat4* invCenteredView, DNmat4* invProjection);

/* Counters accumulated since the last reset (device work must be finished). */
bool DN_get_stats(DNvolume* vol, DNstats* out);
void DN_reset_stats(DNvolume* vol);

/* Copies the FP32 lighting of every loaded chunk to the host:
 * rows (global voxel index, diffuse rgb, specular rgb).  Returns the row
 * count; call with NULL arrays to get the count only. */
size_t DN_export_lighting(DNvolume* vol, uint32_t* index, float* diffuse, float* specular, size_t capacity);
/* Per-tile device state: 0 absent, 1 unloaded, 2 loaded, 3 requested; visible flag; lastUsed; sample count. */
bool DN_export_tiles(DNvolume* vol, uint8_t* state, uint8_t* visible, uint32_t* lastUsed, uint32_t* samples);
/* The request words (tile << 4 | group) of the last DN_sync_gpu, in device order. */
size_t DN_export_requests(DNvolume* vol, uint32_t* out, size_t capacity);

/* A volume with only the CPU-side map (no device state): edit, pick and file
 * operations work; sync, draw and lighting report an error. */
DNvolume* DN_create_volume_cpu(DNuvec3 mapSize, unsigned int minChunks);

/* .voxvol chunk codec (voxel.c:301-518); mem must hold 2 * sizeof(DNchunk)
 * bytes.  Decompress returns 0, or -1 for malformed input. */
size_t DN_compress_chunk(const DNvolume* vol, const DNchunk* chunk, uint8_t* mem);
int DN_decompress_chunk(const DNvolume* vol, const uint8_t* mem, size_t size, DNchunk* chunk);

/* The packing DN_sync_gpu applies to a changed chunk (surface cull, 512-bit occupancy mask, partial
 * counts at 128/256/384, linearised albedo; voxel.c:1397-1461).  words: 2 per surface voxel (normal
 * word, linear albedo word), room for 512 voxels.  Returns the surface voxel count. */
uint32_t dn_pack_chunk(const DNvolume* vol, const DNchunk* chunk, uint32_t mask[16], uint32_t partial[3], uint32_t* words);
/* The surface voxel count of dn_pack_chunk computed the way DN_sync_gpu sizes a chunk's pool range before
 * the device packs it (64-bit occupancy boards; no words written).  Equal to dn_pack_chunk's return value. */
uint32_t dn_count_surface(const DNvolume* vol, const DNchunk* chunk);

/* Struct sizes and field offsets for language bindings; returns the number of entries. */
size_t DN_abi_layout(uint64_t* out, size_t n);

/* Batches: the frame work of many volumes run as kernels that each cover every volume (one draw launch
 * over all images, one sync launch over all maps, one persistent lighting launch over every map's
 * lighting requests), replayed as a CUDA graph while the frame's composition repeats.  Each volume's
 * results are exactly those of calling DN_draw, DN_sync_gpu and DN_update_lighting on it in that order
 * with the same arguments.  A volume added to a batch runs all its device work on the batch's stream.
 * A batch keeps its frames' argument tables (about 11 KB per volume in a frame) in 4 MiB of pinned host
 * memory and 4 MiB of device memory from its first frame on, more only for frames of over about 370
 * volumes. */
typedef struct DNbatch DNbatch;

#define DN_PHASE_DRAW  0x1u
#define DN_PHASE_SYNC  0x2u
#define DN_PHASE_LIGHT 0x4u

typedef struct DNbatchItem
{
	DNvolume* vol;
	unsigned int phases;                 /* DN_PHASE_*: run in the order draw, sync, lighting */
	DNimage* output;                     /* draw: as DN_draw */
	DNmat4 view, projection;
	DNmemOp op;                          /* sync: as DN_sync_gpu */
	int lightingSplit;
	int numDiffuseSamples, maxDiffuseSamples;   /* lighting: as DN_update_lighting */
	float time;
	int rasterColorTexture, rasterDepthTexture; /* draw: as DN_draw (0: none) */
} DNbatchItem;

DNbatch* DN_batch_create(void);
void DN_batch_destroy(DNbatch* batch);
bool DN_batch_add(DNbatch* batch, DNvolume* vol);
bool DN_batch_remove(DNbatch* batch, DNvolume* vol);
/* one frame over the items (each volume at most once, every volume a member) */
bool DN_batch_run(DNbatch* batch, const DNbatchItem* items, unsigned int count);
/* waits for the batch's work; refreshes every member's numLightingRequests */
bool DN_batch_finish(DNbatch* batch);
/* counters of the batch's launches since the last reset */
bool DN_batch_get_stats(DNbatch* batch, DNstats* out);
void DN_batch_reset_stats(DNbatch* batch);
/* picks the batched lighting launch's stream batch and blocks per SM by timing the last frame's
 * lighting under each candidate; results are unaffected */
bool DN_batch_autotune(DNbatch* batch);
/* the CUDA stream (cudaStream_t) all work of the batch and its members runs on */
void* DN_batch_stream(DNbatch* batch);

#ifdef __cplusplus
}
#endif

#endif
