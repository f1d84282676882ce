/*
 * voxel.c -- host side of the DoonEngine DN_* API (include/DoonEngine/voxel.h)
 * on top of the CUDA C ABI (include/dn_cuda.h).
 *
 * The CPU-side map (handles + 8x8x8 chunks) and the voxel edit API keep the
 * reference's semantics (src/DoonEngine/voxel.c:659-714, 1101-1316).  What the
 * reference does with OpenGL is done here as follows:
 *   - chunks changed through the API are recorded in a per-volume dirty list;
 *     DN_sync_gpu packs each changed chunk (surface cull, occupancy mask,
 *     partial counts, linearised albedo: voxel.c:1391-1461) and stages it in
 *     the device pool in one batched upload, instead of packing only chunks
 *     that rays requested (voxel.c:1517-1531).  The device flips a requested
 *     chunk to "loaded" at the next sync exactly when the reference would
 *     upload it, so the observable state sequence is unchanged, and no
 *     per-frame readback of the map is needed (the reference maps the whole
 *     map buffer every frame, voxel.c:731);
 *   - device record slots and voxel ranges come from a host-side allocator
 *     with power-of-two size classes (32..512 voxels) and free lists, in
 *     place of the linear node scan and bubble-sort defragmentation of
 *     voxel.c:1554-1695; the pool grows by doubling before a chunk would not
 *     fit, so every requested chunk loads in the same sync (the reference
 *     fails the upload, doubles at the end of the sync and loads it a frame
 *     later, voxel.c:1592-1596, 773-782).
 */
#include "DoonEngine/voxel.h"
#include "DoonEngine/serve.h"
#include "dn_cuda.h"
#include "dn_residency.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <pthread.h>

/* ------------------------------------------------------------- globals */

void (*g_DN_message_callback)(DNmessageType, DNmessageSeverity, const char*) = NULL;

static DNmallocFn s_malloc = malloc;
static DNfreeFn s_free = free;
static DNreallocFn s_realloc = realloc;

void DN_set_allocator(DNmallocFn m, DNfreeFn f, DNreallocFn r)
{
	s_malloc = m ? m : malloc;
	s_free = f ? f : free;
	s_realloc = r ? r : realloc;
}
void* DN_host_malloc(size_t s) { return s_malloc(s); }
void DN_host_free(void* p) { if (p) s_free(p); }
void* DN_host_realloc(void* p, size_t s) { return s_realloc(p, s); }

static void dn_msg(DNmessageType t, DNmessageSeverity s, const char* fmt, ...)
{
	if (!g_DN_message_callback) return;
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_DN_message_callback(t, s, buf);
}

static int s_initialized = 0;
static uint8_t s_linear[256];   /* sRGB byte -> linear byte, voxel.c:1441-1447 */
static void init_linear_table(void);

#define GET_MATERIAL_ID(x) ((x) >> 24)
#define NUM_CLASSES 5           /* voxel ranges of 32, 64, 128, 256, 512 voxels */

/* ----------------------------------------------------- private volume state */

typedef struct u32vec { uint32_t* v; size_t n, cap; } u32vec;

static int u32_push(u32vec* a, uint32_t x)
{
	if (a->n == a->cap) {
		size_t nc = a->cap ? a->cap * 2 : 256;
		uint32_t* nv = (uint32_t*)DN_REALLOC(a->v, nc * sizeof(uint32_t));
		if (!nv) return 0;
		a->v = nv; a->cap = nc;
	}
	a->v[a->n++] = x;
	return 1;
}

typedef struct DNvolumePriv
{
	DNvolume pub;              /* must stay first */
	uint8_t* dirty;            /* per tile */
	u32vec dirtyList;
	uint32_t* tileSlot;        /* per tile: staged record slot or DN_SLOT_NONE */
	/* record slots */
	uint32_t slotCap, slotNext;
	u32vec freeSlots;
	uint32_t* slotBase;        /* per slot: first voxel */
	uint8_t* slotClass;        /* per slot: size class */
	uint32_t* slotGroups;      /* per slot: ceil(nvox/32) */
	/* voxel ranges */
	uint64_t poolNext;
	u32vec freeRanges[NUM_CLASSES];
	uint64_t groupsStaged;
	uint64_t stagedChunks;
	/* sync scratch */
	dn_tile_op* ops; size_t opsCap;
	dn_chunk_record* recs; size_t recsCap;
	uint32_t* vwords; size_t vwordsCap;   /* in uint32 units; DN_HOST_PACKING only */
	const void** chunkVox; size_t chunkVoxCap;   /* per staged record: its chunk's voxels (packed on the device) */
	dn_pack_params pack;       /* the packing parameters of the sync being prepared */
	int hostPack;              /* DN_HOST_PACKING=1 at creation: records are packed on the host */
	u32vec deferredSlots;
	/* the last view/projection passed to DN_draw */
	float sphereK; float spherePts[64][3]; uint32_t sphereValid;
	struct DNbatch* batch;     /* the batch this volume belongs to, if any */
	uint64_t batchStamp;       /* the batch run that last listed this volume */
	/* residency (DN_set_residency) */
	DNresidency residency;
	uint64_t createChunks;     /* min(tiles, minChunks) of DN_create_volume (voxel.c:181) */
	uint64_t syncs;            /* syncs so far */
	dn_nodes nodes;            /* DN_RESIDENCY_LRU: the reference's voxel buffer nodes */
	uint8_t* lruState;         /* per tile: 0 absent, 1 unloaded, 2 loaded -- the device's, mirrored */
	uint32_t* lruLast;         /* per tile: lastUsed, mirrored */
	uint8_t* lruReq;           /* per tile: requested / touched bytes read back at a sync */
	uint8_t* lruTouch;
	uint32_t* lruOp;           /* per tile: 1 + index of its op in the sync being prepared, 0 for none */
} DNvolumePriv;

static inline DNvolumePriv* priv(DNvolume* v) { return (DNvolumePriv*)v; }

/* ------------------------------------------------------------ init / quit */

bool DN_init(void)
{
	int rc = dn_cuda_init(-1);
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_FATAL, "failed to initialise the CUDA device: %s", dn_cuda_last_error());
		return false;
	}
	init_linear_table();
	s_initialized = 1;
	return true;
}

void DN_quit(void)
{
	dn_cuda_shutdown();
	s_initialized = 0;
}

/* --------------------------------------------------------- create / delete */

static void clear_chunk(DNvolume* vol, size_t index)
{
	/* voxel.c:1353-1363 */
	DNchunk* c = &vol->chunks[index];
	c->pos = (DNivec3){-1, -1, -1};
	c->updated = false;
	c->numVoxels = 0;
	c->numVoxelsGpu = 0;
	for (int x = 0; x < 8; x++)
		for (int y = 0; y < 8; y++)
			for (int z = 0; z < 8; z++) c->voxels[x][y][z].normal = UINT32_MAX;
}

static size_t num_tiles(DNuvec3 s) { return (size_t)s.x * s.y * s.z; }

static void lru_free(DNvolumePriv* p)
{
	dn_nodes_free(&p->nodes);
	DN_FREE(p->lruState); DN_FREE(p->lruLast); DN_FREE(p->lruReq); DN_FREE(p->lruTouch); DN_FREE(p->lruOp);
	p->lruState = NULL; p->lruLast = NULL; p->lruReq = NULL; p->lruTouch = NULL; p->lruOp = NULL;
}

/* the per-tile mirrors of DN_RESIDENCY_LRU, zeroed: every tile absent, lastUsed 0 */
static bool lru_alloc_tiles(DNvolumePriv* p, size_t tiles)
{
	size_t n = tiles ? tiles : 1;
	DN_FREE(p->lruState); DN_FREE(p->lruLast); DN_FREE(p->lruReq); DN_FREE(p->lruTouch); DN_FREE(p->lruOp);
	p->lruState = (uint8_t*)DN_MALLOC(n);
	p->lruLast = (uint32_t*)DN_MALLOC(n * sizeof(uint32_t));
	p->lruReq = (uint8_t*)DN_MALLOC(n);
	p->lruTouch = (uint8_t*)DN_MALLOC(n);
	p->lruOp = (uint32_t*)DN_MALLOC(n * sizeof(uint32_t));
	if (!p->lruState || !p->lruLast || !p->lruReq || !p->lruTouch || !p->lruOp) return false;
	memset(p->lruState, 0, n); memset(p->lruLast, 0, n * sizeof(uint32_t));
	memset(p->lruReq, 0, n); memset(p->lruTouch, 0, n); memset(p->lruOp, 0, n * sizeof(uint32_t));
	return true;
}

static void free_priv_arrays(DNvolumePriv* p)
{
	lru_free(p);
	DN_FREE(p->dirty); DN_FREE(p->dirtyList.v); DN_FREE(p->tileSlot);
	DN_FREE(p->freeSlots.v); DN_FREE(p->slotBase); DN_FREE(p->slotClass); DN_FREE(p->slotGroups);
	for (int c = 0; c < NUM_CLASSES; c++) DN_FREE(p->freeRanges[c].v);
	DN_FREE(p->ops); DN_FREE(p->recs); DN_FREE(p->vwords); DN_FREE(p->chunkVox); DN_FREE(p->deferredSlots.v);
}

static bool alloc_tile_arrays(DNvolumePriv* p, size_t tiles)
{
	p->dirty = (uint8_t*)DN_MALLOC(tiles ? tiles : 1);
	p->tileSlot = (uint32_t*)DN_MALLOC(sizeof(uint32_t) * (tiles ? tiles : 1));
	if (!p->dirty || !p->tileSlot) return false;
	memset(p->dirty, 0, tiles);
	for (size_t i = 0; i < tiles; i++) p->tileSlot[i] = DN_SLOT_NONE;
	return true;
}

static void init_linear_table(void)
{
	for (int b = 0; b < 256; b++) {
		float l = (float)b * 0.00392156862f;
		l = powf(l, DN_GAMMA);
		l = l * 255.0f;
		s_linear[b] = (uint8_t)l;
	}
}

static DNvolume* create_volume(DNuvec3 mapSize, unsigned int minChunks, int withDevice);

DNvolume* DN_create_volume(DNuvec3 mapSize, unsigned int minChunks)
{
	if (!s_initialized && !DN_init()) return NULL;
	return create_volume(mapSize, minChunks, 1);
}

DNvolume* DN_create_volume_cpu(DNuvec3 mapSize, unsigned int minChunks)
{
	init_linear_table();
	return create_volume(mapSize, minChunks, 0);
}

static DNvolume* create_volume(DNuvec3 mapSize, unsigned int minChunks, int withDevice)
{
	size_t tiles = num_tiles(mapSize);
	if (tiles == 0 || tiles >= (1u << 28)) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "invalid map size %ux%ux%u", mapSize.x, mapSize.y, mapSize.z);
		return NULL;
	}
	DNvolumePriv* p = (DNvolumePriv*)DN_MALLOC(sizeof(DNvolumePriv));
	if (!p) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_FATAL, "failed to allocate memory for the volume");
		return NULL;
	}
	memset(p, 0, sizeof(*p));
	DNvolume* vol = &p->pub;
	{
		const char* hp = getenv("DN_HOST_PACKING");
		p->hostPack = hp && atoi(hp) != 0;
	}

	/* sized from x*y*z (the reference sizes its GPU buffers from x*y*x, voxel.c:173, 184) */
	size_t numChunks = tiles < minChunks ? tiles : (size_t)minChunks;
	p->createChunks = numChunks;
	if (numChunks == 0) numChunks = 1;

	vol->map = (DNchunkHandle*)DN_MALLOC(sizeof(DNchunkHandle) * tiles);
	if (!vol->map) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_FATAL, "failed to allocate memory for map"); goto fail; }
	memset(vol->map, 0, sizeof(DNchunkHandle) * tiles);

	vol->chunks = (DNchunk*)DN_MALLOC(sizeof(DNchunk) * numChunks);
	if (!vol->chunks) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_FATAL, "failed to allocate memory for chunks"); goto fail; }
	vol->chunkCap = numChunks;
	for (size_t i = 0; i < numChunks; i++) clear_chunk(vol, i);

	vol->materials = (DNmaterial*)DN_MALLOC(sizeof(DNmaterial) * DN_MAX_MATERIALS);
	if (!vol->materials) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_FATAL, "failed to allocate memory for materials"); goto fail; }
	memset(vol->materials, 0, sizeof(DNmaterial) * DN_MAX_MATERIALS);

	if (!alloc_tile_arrays(p, tiles)) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_FATAL, "failed to allocate memory for tile state"); goto fail; }

	{
		uint32_t slotCap = (uint32_t)(numChunks < 64 ? 64 : numChunks);
		uint64_t voxCap = (uint64_t)DN_CHUNK_LENGTH * numChunks / 2;
		if (voxCap < 4096) voxCap = 4096;
		int rc = withDevice ? dn_cuda_map_create(mapSize.x, mapSize.y, mapSize.z, slotCap, voxCap, &vol->gpu) : DN_CUDA_OK;
		if (rc != DN_CUDA_OK) {
			dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_FATAL, "failed to create the device map: %s", dn_cuda_last_error());
			goto fail;
		}
		p->slotCap = slotCap;
		p->slotBase = (uint32_t*)DN_MALLOC(sizeof(uint32_t) * slotCap);
		p->slotClass = (uint8_t*)DN_MALLOC(slotCap);
		p->slotGroups = (uint32_t*)DN_MALLOC(sizeof(uint32_t) * slotCap);
		if (!p->slotBase || !p->slotClass || !p->slotGroups) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_FATAL, "failed to allocate slot tables"); goto fail; }
		vol->voxelCap = voxCap;
		vol->lightingRequestCap = 1024;   /* the device starts with 1024 request words */
	}

	vol->mapSize = mapSize;
	vol->nextChunk = 0;
	vol->numLightingRequests = 0;
	vol->lightingRequests = NULL;
	vol->gpuVoxelLayout = NULL;

	/* defaults, voxel.c:261-278 */
	vol->camPos = (DNvec3){{0.0f, 0.0f, 0.0f}};
	vol->camOrient = (DNvec3){{0.0f, 0.0f, 0.0f}};
	vol->camFOV = 90.0f;
	vol->camViewMode = 0;
	vol->sunDir = (DNvec3){{1.0f, 1.0f, 1.0f}};
	vol->sunStrength = (DNvec3){{0.6f, 0.6f, 0.6f}};
	vol->ambientLightStrength = (DNvec3){{0.01f, 0.01f, 0.01f}};
	vol->diffuseBounceLimit = 5;
	vol->specBounceLimit = 2;
	vol->shadowSoftness = 10.0f;
	vol->useCubemap = false;
	vol->skyGradientBot = (DNvec3){{0.71f, 0.85f, 0.90f}};
	vol->skyGradientTop = (DNvec3){{0.00f, 0.45f, 0.74f}};
	vol->frameNum = 0;
	vol->lastTime = 123.456f;
	vol->emissiveStrength = 1.0f;
	vol->numDirectRays = 15;
	vol->rngMode = 0;
	vol->mapId = 0;
	vol->truncateDispatch = 0;
	vol->deviceBudgetBytes = 0;
	return vol;

fail:
	if (vol->gpu) dn_cuda_map_destroy(vol->gpu);
	DN_FREE(vol->map); DN_FREE(vol->chunks); DN_FREE(vol->materials);
	free_priv_arrays(p);
	DN_FREE(p);
	return NULL;
}

void DN_delete_volume(DNvolume* vol)
{
	if (!vol) return;
	DNvolumePriv* p = priv(vol);
	if (p->batch) DN_batch_remove(p->batch, vol);
	if (vol->gpu) dn_cuda_map_destroy(vol->gpu);
	DN_FREE(vol->map); DN_FREE(vol->chunks); DN_FREE(vol->materials);
	free_priv_arrays(p);
	DN_FREE(p);
}

/* ------------------------------------------------------------ dirty tiles */

static void mark_dirty(DNvolume* vol, size_t tile)
{
	DNvolumePriv* p = priv(vol);
	if (p->dirty[tile]) return;
	if (!u32_push(&p->dirtyList, (uint32_t)tile)) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to record a changed chunk");
		return;
	}
	p->dirty[tile] = 1;
}

/* marks a chunk read from a file: staged at the next sync, not counted as updated */
void DN_volume_mark_loaded_chunk(DNvolume* vol, size_t tile) { mark_dirty(vol, tile); }

/* ------------------------------------------------------------ chunk memory */

int DN_add_chunk(DNvolume* vol, DNivec3 pos)
{
	/* voxel.c:659-706: ring search from nextChunk for a free chunk, else double the capacity */
	size_t i = vol->nextChunk;
	do {
		if (!DN_in_map_bounds(vol, vol->chunks[i].pos)) {
			size_t mapIndex = DN_FLATTEN_INDEX(pos, vol->mapSize);
			vol->map[mapIndex].chunkIndex = (uint32_t)i;
			vol->map[mapIndex].flag = 1;
			vol->chunks[i].pos = pos;
			vol->nextChunk = (i == vol->chunkCap - 1) ? 0 : i + 1;
			mark_dirty(vol, mapIndex);
			return (int)i;
		}
		i++;
		if (i >= vol->chunkCap) i = 0;
	} while (i != vol->nextChunk);

	size_t tiles = num_tiles(vol->mapSize);
	size_t newCap = vol->chunkCap * 2 < tiles ? vol->chunkCap * 2 : tiles;
	dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_NOTE, "automatically resizing chunk memory to accomodate %zu chunks (%zu bytes)",
	       newCap, newCap * sizeof(DNchunk));
	i = vol->chunkCap;
	if (newCap <= vol->chunkCap || !DN_set_max_chunks(vol, newCap)) return -1;
	size_t mapIndex = DN_FLATTEN_INDEX(pos, vol->mapSize);
	vol->map[mapIndex].chunkIndex = (uint32_t)i;
	vol->map[mapIndex].flag = 1;
	vol->chunks[i].pos = pos;
	vol->nextChunk = (i == vol->chunkCap - 1) ? 0 : i + 1;
	mark_dirty(vol, mapIndex);
	return (int)i;
}

void DN_remove_chunk(DNvolume* vol, DNivec3 pos)
{
	/* voxel.c:708-714 */
	size_t mapIndex = DN_FLATTEN_INDEX(pos, vol->mapSize);
	vol->map[mapIndex].flag = 0;
	vol->nextChunk = vol->map[mapIndex].chunkIndex;
	clear_chunk(vol, vol->map[mapIndex].chunkIndex);
	mark_dirty(vol, mapIndex);
}

/* ------------------------------------------------------------- settings */

bool DN_set_max_chunks(DNvolume* vol, size_t num)
{
	/* voxel.c:1012-1029 */
	DNchunk* nc = (DNchunk*)DN_REALLOC(vol->chunks, sizeof(DNchunk) * num);
	if (!nc) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate memory for chunks");
		return false;
	}
	vol->chunks = nc;
	for (size_t i = vol->chunkCap; i < num; i++) clear_chunk(vol, i);
	vol->chunkCap = num;
	return true;
}

static bool need_device(DNvolume* vol, const char* what)
{
	if (vol->gpu) return true;
	dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "%s: this volume has no device state (created with DN_create_volume_cpu)", what);
	return false;
}

static bool ensure_slots(DNvolumePriv* p, uint32_t need)
{
	if (need <= p->slotCap) return true;
	uint32_t nc = p->slotCap;
	while (nc < need) nc *= 2;
	uint32_t* b = (uint32_t*)DN_REALLOC(p->slotBase, sizeof(uint32_t) * nc);
	if (b) p->slotBase = b;
	uint8_t* c = (uint8_t*)DN_REALLOC(p->slotClass, nc);
	if (c) p->slotClass = c;
	uint32_t* g = (uint32_t*)DN_REALLOC(p->slotGroups, sizeof(uint32_t) * nc);
	if (g) p->slotGroups = g;
	if (!b || !c || !g) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to grow the slot tables");
		return false;
	}
	int rc = dn_cuda_reserve(p->pub.gpu, nc, 0, 0);
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to grow the device chunk records: %s", dn_cuda_last_error());
		return false;
	}
	p->slotCap = nc;
	return true;
}

/* grows the device pool keeping its contents */
static bool pool_reserve(DNvolume* vol, size_t num)
{
	if (num <= vol->voxelCap) return true;
	if (!need_device(vol, "DN_set_max_voxels_gpu")) return false;
	int rc = dn_cuda_reserve(vol->gpu, 0, num, 0);
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate voxel buffer: %s", dn_cuda_last_error());
		return false;
	}
	vol->voxelCap = num;
	return true;
}

bool DN_set_max_voxels_gpu(DNvolume* vol, size_t num)
{
	/* voxel.c:1031-1082.  The device pool only grows; with DN_RESIDENCY_LRU the node buffer grows too */
	DNvolumePriv* p = priv(vol);
	if (!pool_reserve(vol, num)) return false;
	if (p->residency == DN_RESIDENCY_LRU && !dn_nodes_grow(&p->nodes, num)) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate memory for GPU voxel layout");
		return false;
	}
	return true;
}

bool DN_set_residency(DNvolume* vol, DNresidency mode)
{
	if (!vol) return false;
	DNvolumePriv* p = priv(vol);
	if (mode == p->residency) return true;
	if (mode != DN_RESIDENCY_KEEP && mode != DN_RESIDENCY_LRU) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "DN_set_residency: unknown mode %d", (int)mode);
		return false;
	}
	if (p->syncs) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "DN_set_residency: set it before the volume's first DN_sync_gpu");
		return false;
	}
	if (p->batch) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "DN_set_residency: the volume belongs to a batch");
		return false;
	}
	if (mode == DN_RESIDENCY_LRU) {
		if (!dn_nodes_init(&p->nodes, p->createChunks) || !lru_alloc_tiles(p, num_tiles(vol->mapSize))) {
			lru_free(p);
			dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate memory for GPU voxel layout");
			return false;
		}
	} else {
		lru_free(p);
	}
	p->residency = mode;
	return true;
}

DNresidency DN_get_residency(const DNvolume* vol)
{
	return vol ? ((const DNvolumePriv*)vol)->residency : DN_RESIDENCY_KEEP;
}

size_t DN_residency_nodes(const DNvolume* vol, size_t* voxelCap, uint32_t* sizes, uint64_t* starts, int64_t* tiles,
                          size_t capacity)
{
	const DNvolumePriv* p = (const DNvolumePriv*)vol;
	if (voxelCap) *voxelCap = 0;
	if (!p || p->residency != DN_RESIDENCY_LRU) return 0;
	if (voxelCap) *voxelCap = (size_t)p->nodes.voxelCap;
	for (size_t i = 0; i < p->nodes.n && i < capacity; i++) {
		if (sizes) sizes[i] = p->nodes.v[i].size;
		if (starts) starts[i] = p->nodes.v[i].start;
		if (tiles) tiles[i] = p->nodes.v[i].tile;
	}
	return p->nodes.n;
}

bool DN_set_max_lighting_requests(DNvolume* vol, size_t num)
{
	/* voxel.c:1084-1096 (request words now live on the device) */
	if (num <= vol->lightingRequestCap) return true;
	if (!need_device(vol, "DN_set_max_lighting_requests")) return false;
	int rc = dn_cuda_reserve(vol->gpu, 0, 0, num);
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to resize lighting request buffer: %s", dn_cuda_last_error());
		return false;
	}
	vol->lightingRequestCap = num;
	return true;
}

static void release_all_slots(DNvolumePriv* p)
{
	p->slotNext = 0;
	p->freeSlots.n = 0;
	p->poolNext = 0;
	for (int c = 0; c < NUM_CLASSES; c++) p->freeRanges[c].n = 0;
	p->groupsStaged = 0;
	p->stagedChunks = 0;
	p->deferredSlots.n = 0;
}

bool DN_set_map_size(DNvolume* vol, DNuvec3 size)
{
	/* voxel.c:957-1010.  The device map restarts with every tile absent and
	 * every existing chunk is re-staged at the next sync (the reference
	 * re-creates its GPU buffers from the CPU handle array, which leaves
	 * them in an undefined state). */
	DNvolumePriv* p = priv(vol);
	size_t tiles = num_tiles(size);
	if (tiles == 0 || tiles >= (1u << 28)) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "invalid map size");
		return false;
	}
	DNchunkHandle* nm = (DNchunkHandle*)DN_MALLOC(sizeof(DNchunkHandle) * tiles);
	uint8_t* nd = (uint8_t*)DN_MALLOC(tiles);
	uint32_t* ns = (uint32_t*)DN_MALLOC(sizeof(uint32_t) * tiles);
	if (!nm || !nd || !ns) {
		DN_FREE(nm); DN_FREE(nd); DN_FREE(ns);
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate memory for map");
		return false;
	}
	for (uint32_t z = 0; z < size.z; z++)
	for (uint32_t y = 0; y < size.y; y++)
	for (uint32_t x = 0; x < size.x; x++) {
		DNivec3 pos = {(int32_t)x, (int32_t)y, (int32_t)z};
		size_t ni = DN_FLATTEN_INDEX(pos, size);
		if (DN_in_map_bounds(vol, pos)) nm[ni] = vol->map[DN_FLATTEN_INDEX(pos, vol->mapSize)];
		else { nm[ni].flag = 0; nm[ni].chunkIndex = 0; }
	}
	int rc = vol->gpu ? dn_cuda_map_resize(vol->gpu, size.x, size.y, size.z) : DN_CUDA_OK;
	if (rc != DN_CUDA_OK) {
		DN_FREE(nm); DN_FREE(nd); DN_FREE(ns);
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate map buffer: %s", dn_cuda_last_error());
		return false;
	}
	DN_FREE(vol->map); DN_FREE(p->dirty); DN_FREE(p->tileSlot);
	vol->map = nm; p->dirty = nd; p->tileSlot = ns;
	vol->mapSize = size;
	for (size_t i = 0; i < vol->chunkCap; i++)
		if (!DN_in_map_bounds(vol, vol->chunks[i].pos)) clear_chunk(vol, i);
	memset(p->dirty, 0, tiles);
	for (size_t i = 0; i < tiles; i++) p->tileSlot[i] = DN_SLOT_NONE;
	p->dirtyList.n = 0;
	release_all_slots(p);
	if (p->residency == DN_RESIDENCY_LRU) {
		/* every tile restarts absent: the nodes are freed with the map (the reference keeps their old
		 * chunk positions, voxel.c:957-1010) */
		for (size_t i = 0; i < p->nodes.n; i++) p->nodes.v[i].tile = -1;
		if (!lru_alloc_tiles(p, tiles)) {
			dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate the residency state");
			lru_free(p);
			p->residency = DN_RESIDENCY_KEEP;
		}
	}
	for (size_t t = 0; t < tiles; t++) if (vol->map[t].flag) mark_dirty(vol, t);
	return true;
}

/* ------------------------------------------------------------ map utility */

bool DN_in_map_bounds(DNvolume* vol, DNivec3 pos)
{
	return pos.x >= 0 && pos.y >= 0 && pos.z >= 0 &&
	       (uint32_t)pos.x < vol->mapSize.x && (uint32_t)pos.y < vol->mapSize.y && (uint32_t)pos.z < vol->mapSize.z;
}

bool DN_in_chunk_bounds(DNivec3 pos)
{
	return pos.x < DN_CHUNK_SIZE && pos.y < DN_CHUNK_SIZE && pos.z < DN_CHUNK_SIZE && pos.x >= 0 && pos.y >= 0 && pos.z >= 0;
}

DNvoxel DN_get_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos)
{
	return DN_decompress_voxel(DN_get_compressed_voxel(vol, mapPos, chunkPos));
}

DNcompressedVoxel DN_get_compressed_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos)
{
	/* voxel.c:1116-1119; a tile without a chunk reads as empty instead of a stale chunk */
	DNchunkHandle h = vol->map[DN_FLATTEN_INDEX(mapPos, vol->mapSize)];
	if (!h.flag) { DNcompressedVoxel e = {UINT32_MAX, 0}; return e; }
	return vol->chunks[h.chunkIndex].voxels[chunkPos.x][chunkPos.y][chunkPos.z];
}

void DN_set_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos, DNvoxel voxel)
{
	DN_set_compressed_voxel(vol, mapPos, chunkPos, DN_compress_voxel(voxel));
}

void DN_set_compressed_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos, DNcompressedVoxel voxel)
{
	/* voxel.c:1126-1161 */
	size_t mapIndex = DN_FLATTEN_INDEX(mapPos, vol->mapSize);
	if (vol->map[mapIndex].flag == 0) {
		if (GET_MATERIAL_ID(voxel.normal) == DN_MATERIAL_EMPTY) return;
		if (DN_add_chunk(vol, mapPos) < 0) return;
	}
	uint32_t chunkIndex = vol->map[mapIndex].chunkIndex;
	DNchunk* c = &vol->chunks[chunkIndex];
	uint32_t oldMat = GET_MATERIAL_ID(c->voxels[chunkPos.x][chunkPos.y][chunkPos.z].normal);
	uint32_t newMat = GET_MATERIAL_ID(voxel.normal);
	if (oldMat == DN_MATERIAL_EMPTY && newMat != DN_MATERIAL_EMPTY)
		c->numVoxels++;
	else if (oldMat != DN_MATERIAL_EMPTY && newMat == DN_MATERIAL_EMPTY) {
		c->numVoxels--;
		if (c->numVoxels <= 0) {
			DN_remove_chunk(vol, mapPos);
			return;
		}
	}
	c->voxels[chunkPos.x][chunkPos.y][chunkPos.z] = voxel;
	c->updated = 1;
	mark_dirty(vol, mapIndex);
}

void DN_remove_voxel(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos)
{
	/* voxel.c:1163-1182 (a tile without a chunk is left alone instead of editing a stale chunk) */
	size_t mapIndex = DN_FLATTEN_INDEX(mapPos, vol->mapSize);
	if (!vol->map[mapIndex].flag) return;
	uint32_t chunkIndex = vol->map[mapIndex].chunkIndex;
	if (DN_does_voxel_exist(vol, mapPos, chunkPos)) {
		vol->chunks[chunkIndex].numVoxels--;
		if (vol->chunks[chunkIndex].numVoxels <= 0) {
			DN_remove_chunk(vol, mapPos);
			return;
		}
	}
	vol->chunks[chunkIndex].voxels[chunkPos.x][chunkPos.y][chunkPos.z].normal = UINT32_MAX;
	vol->chunks[chunkIndex].updated = 1;
	mark_dirty(vol, mapIndex);
}

bool DN_does_chunk_exist(DNvolume* vol, DNivec3 pos)
{
	return vol->map[DN_FLATTEN_INDEX(pos, vol->mapSize)].flag >= 1;
}

bool DN_does_voxel_exist(DNvolume* vol, DNivec3 mapPos, DNivec3 chunkPos)
{
	return GET_MATERIAL_ID(DN_get_compressed_voxel(vol, mapPos, chunkPos).normal) != DN_MATERIAL_EMPTY;
}

#define SIGNF(n) (((n) > 0) ? 1 : (((n) < 0) ? -1 : 0))

bool DN_step_map(DNvolume* vol, DNvec3 rayDir, DNvec3 rayPos, int maxSteps, DNivec3* hitPos, DNvoxel* hitVoxel, DNivec3* hitNormal)
{
	/* CPU picking ray, voxel.c:1195-1272: single-level voxel DDA with strict
	 * '<' ties; the starting side distances are evaluated in double and
	 * rounded to float, as the reference's expression does. */
	*hitNormal = (DNivec3){-1000, -1000, -1000};
	rayPos = DN_vec3_scale(rayPos, (float)DN_CHUNK_SIZE);
	DNvec3 inv = {{1 / rayDir.x, 1 / rayDir.y, 1 / rayDir.z}};
	DNvec3 sgn = {{(float)SIGNF(rayDir.x), (float)SIGNF(rayDir.y), (float)SIGNF(rayDir.z)}};
	DNivec3 pos = {(int32_t)floor(rayPos.x), (int32_t)floor(rayPos.y), (int32_t)floor(rayPos.z)};
	DNvec3 delta = {{fabsf(inv.x), fabsf(inv.y), fabsf(inv.z)}};
	DNivec3 step = {(int32_t)sgn.x, (int32_t)sgn.y, (int32_t)sgn.z};
	DNvec3 side;
	side.x = (float)(((double)(sgn.x * ((float)pos.x - rayPos.x)) + (double)sgn.x * 0.5 + 0.5) * (double)delta.x);
	side.y = (float)(((double)(sgn.y * ((float)pos.y - rayPos.y)) + (double)sgn.y * 0.5 + 0.5) * (double)delta.y);
	side.z = (float)(((double)(sgn.z * ((float)pos.z - rayPos.z)) + (double)sgn.z * 0.5 + 0.5) * (double)delta.z);
	for (int n = 0; n < maxSteps; n++) {
		DNivec3 mp, cp;
		DN_separate_position(pos, &mp, &cp);
		if (pos.x < 0) mp.x--;
		if (pos.y < 0) mp.y--;
		if (pos.z < 0) mp.z--;
		if (DN_in_map_bounds(vol, mp) && DN_does_chunk_exist(vol, mp) && DN_does_voxel_exist(vol, mp, cp)) {
			*hitVoxel = DN_get_voxel(vol, mp, cp);
			*hitPos = pos;
			return true;
		}
		if (side.x < side.y) {
			if (side.x < side.z) { side.x += delta.x; pos.x += step.x; *hitNormal = (DNivec3){-step.x, 0, 0}; }
			else { side.z += delta.z; pos.z += step.z; *hitNormal = (DNivec3){0, 0, -step.z}; }
		} else {
			if (side.y < side.z) { side.y += delta.y; pos.y += step.y; *hitNormal = (DNivec3){0, -step.y, 0}; }
			else { side.z += delta.z; pos.z += step.z; *hitNormal = (DNivec3){0, 0, -step.z}; }
		}
	}
	return false;
}

void DN_separate_position(DNivec3 pos, DNivec3* mapPos, DNivec3* chunkPos)
{
	*mapPos = (DNivec3){pos.x / DN_CHUNK_SIZE, pos.y / DN_CHUNK_SIZE, pos.z / DN_CHUNK_SIZE};
	*chunkPos = (DNivec3){pos.x % DN_CHUNK_SIZE, pos.y % DN_CHUNK_SIZE, pos.z % DN_CHUNK_SIZE};
}

DNvec3 DN_cam_dir(DNvec3 orient)
{
	DNmat3 r = DN_mat4_top_left(DN_mat4_rotate_euler(orient));
	return DN_mat3_mult_vec3(r, (DNvec3){{0.0f, 0.0f, 1.0f}});
}

DNcompressedVoxel DN_compress_voxel(DNvoxel voxel)
{
	/* voxel.c:1289-1301 */
	DNcompressedVoxel res;
	uint32_t nb[3];
	for (int i = 0; i < 3; i++) {
		float n = voxel.normal.v[i];
		n = n < 1.0f ? n : 1.0f;
		n = n > -1.0f ? n : -1.0f;
		nb[i] = (uint32_t)(((int)(n * 255.0f) + 255) / 2);
	}
	res.normal = ((uint32_t)voxel.material << 24) | (nb[0] << 16) | (nb[1] << 8) | nb[2];
	res.albedo = ((uint32_t)voxel.albedo.r << 24) | ((uint32_t)voxel.albedo.g << 16) | ((uint32_t)voxel.albedo.b << 8);
	return res;
}

DNvoxel DN_decompress_voxel(DNcompressedVoxel voxel)
{
	/* voxel.c:1303-1316 */
	DNvoxel res;
	const float inv255 = 1.0f / 255.0f;
	int32_t nx = (int32_t)((voxel.normal >> 16) & 0xFF) * 2 - 255;
	int32_t ny = (int32_t)((voxel.normal >> 8) & 0xFF) * 2 - 255;
	int32_t nz = (int32_t)(voxel.normal & 0xFF) * 2 - 255;
	res.normal.x = (float)nx * inv255;
	res.normal.y = (float)ny * inv255;
	res.normal.z = (float)nz * inv255;
	res.material = (uint8_t)(voxel.normal >> 24);
	res.albedo.r = (uint8_t)((voxel.albedo >> 24) & 0xFF);
	res.albedo.g = (uint8_t)((voxel.albedo >> 16) & 0xFF);
	res.albedo.b = (uint8_t)((voxel.albedo >> 8) & 0xFF);
	return res;
}

/* --------------------------------------------------------------- packing */

static inline int face_visible(const DNvolume* vol, const DNchunk* c, int x, int y, int z)
{
	/* voxel.c:1391-1394 */
	if (x < 0 || y < 0 || z < 0 || x >= 8 || y >= 8 || z >= 8) return 1;
	uint32_t m = GET_MATERIAL_ID(c->voxels[x][y][z].normal);
	return m == DN_MATERIAL_EMPTY || vol->materials[m].opacity < 1.0f;
}

/* surface cull + occupancy mask + partial counts + linear albedo (voxel.c:1397-1461);
 * writes the voxel words (2 per voxel) to out and returns the voxel count */
static uint32_t pack_chunk(const DNvolume* vol, const DNchunk* c, dn_chunk_record* rec, uint32_t* out)
{
	memset(rec->mask, 0, sizeof(rec->mask));
	memset(rec->partial, 0, sizeof(rec->partial));
	uint32_t n = 0;
	for (int z = 0; z < 8; z++)
	for (int y = 0; y < 8; y++)
	for (int x = 0; x < 8; x++) {
		uint32_t idx = (uint32_t)(x + 8 * (y + 8 * z));
		if (idx == 128 || idx == 256 || idx == 384) rec->partial[(idx >> 7) - 1] = n;
		uint32_t nw = c->voxels[x][y][z].normal;
		if (GET_MATERIAL_ID(nw) == DN_MATERIAL_EMPTY) continue;
		if (!(face_visible(vol, c, x + 1, y, z) || face_visible(vol, c, x - 1, y, z) ||
		      face_visible(vol, c, x, y + 1, z) || face_visible(vol, c, x, y - 1, z) ||
		      face_visible(vol, c, x, y, z + 1) || face_visible(vol, c, x, y, z - 1))) continue;
		rec->mask[idx >> 5] |= 1u << (idx & 31);
		uint32_t a = c->voxels[x][y][z].albedo;
		uint32_t r = s_linear[(a >> 24) & 0xFF], g = s_linear[(a >> 16) & 0xFF], b = s_linear[(a >> 8) & 0xFF];
		out[2 * n] = nw;
		out[2 * n + 1] = (r << 24) | (g << 16) | (b << 8);
		n++;
	}
	rec->nvox = n;
	return n;
}

/* the materials a face is seen through at this sync (voxel.c:1391-1394): empty, or opacity < 1 */
static void pack_params(const DNvolume* vol, dn_pack_params* pk)
{
	memset(pk->seeThrough, 0, sizeof(pk->seeThrough));
	for (uint32_t m = 0; m < DN_MAX_MATERIALS; m++)
		if (m == DN_MATERIAL_EMPTY || vol->materials[m].opacity < 1.0f) pk->seeThrough[m >> 5] |= 1u << (m & 31);
	memcpy(pk->linear, s_linear, sizeof(pk->linear));
}

/* The number of voxels pack_chunk keeps: the same cull on 64-bit boards of the chunk's [x][y][z] storage,
 * word x holding bit 8*y + z, so one shift tests a face neighbour of 64 voxels at once.  The device packs
 * the chunk itself (dn_cuda_sync_chunks); the host needs only this count to size the chunk's pool range. */
static uint32_t count_kept(const DNchunk* c, const uint32_t see[8])
{
	uint64_t solid[8], thru[8];
	for (int x = 0; x < 8; x++) {
		const DNcompressedVoxel* v = &c->voxels[x][0][0];
		uint64_t sb = 0, tb = 0;
		for (int i = 0; i < 64; i++) {
			const uint32_t m = GET_MATERIAL_ID(v[i].normal);
			sb |= (uint64_t)(m != DN_MATERIAL_EMPTY) << i;
			tb |= (uint64_t)((see[m >> 5] >> (m & 31)) & 1u) << i;
		}
		solid[x] = sb; thru[x] = tb;
	}
	uint32_t n = 0;
	for (int x = 0; x < 8; x++) {
		const uint64_t t = thru[x];
		/* a neighbour outside the chunk counts as see-through: z = 7 and z = 0 are bits 7 and 0 of each
		 * byte, y = 7 and y = 0 the top and bottom byte, x = 7 and x = 0 the last and first word */
		uint64_t nb = (t >> 1) | 0x8080808080808080ull;   /* z + 1 */
		nb |= (t << 1) | 0x0101010101010101ull;           /* z - 1 */
		nb |= (t >> 8) | 0xFF00000000000000ull;           /* y + 1 */
		nb |= (t << 8) | 0x00000000000000FFull;           /* y - 1 */
		nb |= x < 7 ? thru[x + 1] : ~0ull;
		nb |= x > 0 ? thru[x - 1] : ~0ull;
		n += (uint32_t)__builtin_popcountll(solid[x] & nb);
	}
	return n;
}

/* ---------------------------------------------------- slot / range allocator */

static uint32_t class_of(uint32_t nvox)
{
	uint32_t c = 0, s = 32;
	while (s < nvox) { s <<= 1; c++; }
	return c;
}

static bool alloc_slot(DNvolumePriv* p, uint32_t nvox, uint32_t* slotOut)
{
	uint32_t slot;
	if (p->freeSlots.n) slot = p->freeSlots.v[--p->freeSlots.n];
	else {
		if (!ensure_slots(p, p->slotNext + 1)) return false;
		slot = p->slotNext++;
	}
	uint32_t cls = class_of(nvox);
	uint64_t base;
	if (p->freeRanges[cls].n) base = p->freeRanges[cls].v[--p->freeRanges[cls].n];
	else {
		uint64_t size = 32ull << cls;
		if (p->poolNext + size > p->pub.voxelCap) {
			uint64_t nc = p->pub.voxelCap ? p->pub.voxelCap : 4096;
			while (p->poolNext + size > nc) nc *= 2;
			dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_NOTE, "automatically resizing voxel buffer to accomodate %llu GPU voxels (%llu bytes)",
			       (unsigned long long)nc, (unsigned long long)(nc * 40));
			if (!pool_reserve(&p->pub, nc)) { u32_push(&p->freeSlots, slot); return false; }
		}
		base = p->poolNext;
		p->poolNext += size;
	}
	p->slotBase[slot] = (uint32_t)base;
	p->slotClass[slot] = (uint8_t)cls;
	p->slotGroups[slot] = (nvox + 31) / 32;
	p->groupsStaged += p->slotGroups[slot];
	p->stagedChunks++;
	*slotOut = slot;
	return true;
}

static void free_slot(DNvolumePriv* p, uint32_t slot)
{
	u32_push(&p->freeRanges[p->slotClass[slot]], p->slotBase[slot]);
	u32_push(&p->freeSlots, slot);
	p->groupsStaged -= p->slotGroups[slot];
	p->stagedChunks--;
}

static bool grow_scratch(void** buf, size_t* cap, size_t need, size_t elem)
{
	if (need <= *cap) return true;
	size_t nc = *cap ? *cap : 64;
	while (nc < need) nc *= 2;
	void* nb = DN_REALLOC(*buf, nc * elem);
	if (!nb) return false;
	*buf = nb; *cap = nc;
	return true;
}

/* ---------------------------------------------------------------- sync */

/* room for one more staged record: record 'nrecs', with its words from vwords[nvw] when packed here */
static bool grow_stage(DNvolumePriv* p, size_t nrecs, uint64_t nvw)
{
	if (!grow_scratch((void**)&p->recs, &p->recsCap, nrecs + 1, sizeof(dn_chunk_record))) return false;
	if (p->hostPack) return grow_scratch((void**)&p->vwords, &p->vwordsCap, (size_t)nvw + 1024, sizeof(uint32_t));
	return grow_scratch((void**)&p->chunkVox, &p->chunkVoxCap, nrecs + 1, sizeof(void*));
}

/* record 'ri' of the sync for chunk c: packed here with DN_HOST_PACKING (its words to vwords[nvw]), else only
 * counted here and packed on the device from the chunk's voxels.  Returns the kept-voxel count. */
static uint32_t stage_record(DNvolume* vol, const DNchunk* c, uint32_t ri, uint64_t nvw)
{
	DNvolumePriv* p = priv(vol);
	dn_chunk_record* r = &p->recs[ri];
	if (p->hostPack) return pack_chunk(vol, c, r, &p->vwords[nvw]);
	memset(r, 0, sizeof(*r));
	r->nvox = count_kept(c, p->pack.seeThrough);
	p->chunkVox[ri] = &c->voxels[0][0][0];
	return r->nvox;
}

/* the device half of a sync prepared by sync_prepare (per-tile pass included unless stageOnly) */
static int sync_issue(DNvolume* vol, const dn_sync_params* sp, uint32_t nops, uint32_t nrecs, uint64_t nvw, int stageOnly)
{
	DNvolumePriv* p = priv(vol);
	if (p->hostPack)
		return stageOnly ? dn_cuda_sync_stage(vol->gpu, p->ops, nops, p->recs, nrecs, p->vwords, nvw / 2)
		                 : dn_cuda_sync(vol->gpu, sp, p->ops, nops, p->recs, nrecs, p->vwords, nvw / 2);
	return stageOnly ? dn_cuda_sync_stage_chunks(vol->gpu, &p->pack, p->ops, nops, p->recs, nrecs, p->chunkVox)
	                 : dn_cuda_sync_chunks(vol->gpu, sp, &p->pack, p->ops, nops, p->recs, nrecs, p->chunkVox);
}

/* the op of tile t in the sync being prepared, appended (with 'flags') when the tile has none; -1 when
 * the scratch cannot grow */
static long lru_op(DNvolumePriv* p, uint32_t t, uint32_t* nops, uint32_t flags)
{
	if (p->lruOp[t]) return (long)p->lruOp[t] - 1;
	if (!grow_scratch((void**)&p->ops, &p->opsCap, (size_t)*nops + 1, sizeof(dn_tile_op))) return -1;
	dn_tile_op* o = &p->ops[*nops];
	o->tile = t; o->flags = flags; o->slot = DN_SLOT_NONE; o->recordIndex = 0;
	p->lruOp[t] = ++*nops;
	return (long)*nops - 1;
}

/* DN_RESIDENCY_LRU: the per-tile loop of DN_sync_gpu (voxel.c:738-762) on the host's node model, in the
 * reference's tile order -- lastUsed, the state machine of _DN_stream_to_gpu (1491-1536) and the node
 * choice of _DN_stream_voxels (1554-1630) -- then the node sort and the buffer growth (764-781).  The
 * decisions reach the device as tile-op bits.  A chunk that loads without a record slot (it was
 * evicted) is packed and staged again, as the reference uploads it again. */
static bool lru_pass(DNvolume* vol, DNmemOp op, uint32_t* nops, uint32_t* nrecs, uint64_t* nvw)
{
	DNvolumePriv* p = priv(vol);
	const size_t tiles = num_tiles(vol->mapSize);
	if (dn_cuda_read_tile_flags(vol->gpu, p->lruReq, p->lruTouch) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to read the tile flags: %s", dn_cuda_last_error());
		return false;
	}
	/* the rays' lastUsed = 0 (voxelShared.comp:143-144) happened before the sync's increments */
	for (size_t t = 0; t < tiles; t++) if (p->lruTouch[t]) p->lruLast[t] = 0;
	for (uint32_t k = 0; k < *nops; k++) p->lruOp[p->ops[k].tile] = k + 1;
	bool grow = false, ok = true;
	for (uint32_t t = 0; t < (uint32_t)tiles && ok; t++) {
		if (p->lruLast[t] != UINT32_MAX) p->lruLast[t]++;
		if (op == DN_READ) continue;
		uint32_t g = p->lruState[t];
		if (g == 1 && p->lruReq[t]) g = 3;
		const bool exists = vol->map[t].flag != 0;
		const bool updated = p->lruOp[t] && (p->ops[p->lruOp[t] - 1].flags & DN_PEND_UPDATED);
		if (exists && g == 0) g = 1;
		else if (!exists && g != 0) { if (g == 2) dn_nodes_unload(&p->nodes, t); g = 0; }
		if (g == 2 && updated) { dn_nodes_unload(&p->nodes, t); g = 3; }
		if (g == 3 && exists) {
			DNchunk* c = &vol->chunks[vol->map[t].chunkIndex];
			p->lruLast[t] = 0;
			int64_t victim = -1;
			int r = dn_nodes_stream(&p->nodes, t, c->numVoxelsGpu, p->lruLast, &victim);
			if (r < 0) {
				dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate memory for GPU voxel layout");
				ok = false;
				r = 0;
			}
			if (r > 0 && victim >= 0) {
				/* the node's chunk is unloaded; if it comes later in the loop it meets its turn unloaded */
				const uint32_t v = (uint32_t)victim;
				long vi = lru_op(p, v, nops, 0);
				if (vi < 0) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate sync scratch"); ok = false; }
				else p->ops[vi].flags |= (v < t) ? DN_PEND_EVICT : DN_PEND_EVICTED;
				p->lruState[v] = 1;
				if (p->tileSlot[v] != DN_SLOT_NONE) { u32_push(&p->deferredSlots, p->tileSlot[v]); p->tileSlot[v] = DN_SLOT_NONE; }
			}
			bool staged = true;
			if (r > 0 && p->tileSlot[t] == DN_SLOT_NONE) {
				/* loads without a record (it was evicted): pack and stage it again */
				staged = false;
				long oi = lru_op(p, t, nops, DN_PEND_VALID | DN_PEND_EXISTS);
				uint32_t slot;
				if (oi < 0 || !grow_stage(p, *nrecs, *nvw)) {
					dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate sync scratch");
					ok = false;
				} else {
					dn_chunk_record* rec = &p->recs[*nrecs];
					uint32_t n = stage_record(vol, c, *nrecs, *nvw);
					if (!alloc_slot(p, n, &slot)) {
						dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to stage a chunk on the device");
					} else {
						rec->pos[0] = c->pos.x; rec->pos[1] = c->pos.y; rec->pos[2] = c->pos.z;
						rec->voxBase = p->slotBase[slot];
						c->numVoxelsGpu = n;
						dn_tile_op* o = &p->ops[oi];
						o->flags |= DN_PEND_VALID | DN_PEND_EXISTS | DN_PEND_STAGED;
						o->slot = slot;
						o->recordIndex = *nrecs;
						p->tileSlot[t] = slot;
						(*nrecs)++;
						*nvw += 2ull * n;
						staged = true;
					}
				}
				if (!staged) dn_nodes_unload(&p->nodes, t);   /* it cannot load after all: the node is free again */
			}
			if (r > 0 && staged) {
				g = 2;
			} else {
				/* no node: unloaded again, and the buffer doubles after the loop */
				g = 1;
				if (r == 0 && ok) grow = true;
				long oi = lru_op(p, t, nops, 0);
				if (oi < 0) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate sync scratch"); ok = false; }
				else p->ops[oi].flags |= DN_PEND_HOLD;
			}
		}
		p->lruState[t] = (uint8_t)g;
	}
	for (uint32_t k = 0; k < *nops; k++) p->lruOp[p->ops[k].tile] = 0;
	if (!ok) return false;
	dn_nodes_sort(&p->nodes, 10);
	if (grow) {
		uint64_t nc = p->nodes.voxelCap * 2, lim = (uint64_t)vol->chunkCap * DN_CHUNK_LENGTH;
		if (nc > lim) nc = lim;
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_NOTE, "automatically resizing voxel buffer to accomodate %llu GPU voxels (%llu bytes)",
		       (unsigned long long)nc, (unsigned long long)(nc * 16));
		if (!dn_nodes_grow(&p->nodes, nc)) {
			dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to reallocate memory for GPU voxel layout");
			return false;
		}
	}
	return true;
}

/* Host half of DN_sync_gpu (voxel.c:719-786): advances frameNum, packs every dirty chunk into the
 * volume's op / record / voxel-word scratch and fills sp.  Returns false when the scratch cannot grow. */
static bool sync_prepare(DNvolume* vol, DNmemOp op, int lightingSplit, dn_sync_params* spOut, uint32_t* nopsOut,
                         uint32_t* nrecsOut, uint64_t* nvwOut)
{
	DNvolumePriv* p = priv(vol);
	if (lightingSplit < 1) lightingSplit = 1;
	vol->frameNum++;
	if (vol->frameNum >= (uint32_t)lightingSplit) vol->frameNum = 0;

	size_t nd = p->dirtyList.n;
	if (!grow_scratch((void**)&p->ops, &p->opsCap, nd ? nd : 1, sizeof(dn_tile_op)) ||
	    !grow_scratch((void**)&p->recs, &p->recsCap, nd ? nd : 1, sizeof(dn_chunk_record)) ||
	    !(p->hostPack ? grow_scratch((void**)&p->vwords, &p->vwordsCap, (nd ? nd : 1) * 1024, sizeof(uint32_t))
	                  : grow_scratch((void**)&p->chunkVox, &p->chunkVoxCap, nd ? nd : 1, sizeof(void*)))) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate sync scratch");
		return false;
	}
	pack_params(vol, &p->pack);
	uint32_t nops = 0, nrecs = 0;
	uint64_t nvw = 0;
	p->deferredSlots.n = 0;
	if (op != DN_READ) {
		for (size_t k = 0; k < nd; k++) {
			uint32_t t = p->dirtyList.v[k];
			p->dirty[t] = 0;
			dn_tile_op* o = &p->ops[nops++];
			o->tile = t;
			o->flags = DN_PEND_VALID;
			o->slot = DN_SLOT_NONE;
			o->recordIndex = 0;
			if (p->tileSlot[t] != DN_SLOT_NONE) u32_push(&p->deferredSlots, p->tileSlot[t]);
			p->tileSlot[t] = DN_SLOT_NONE;
			if (vol->map[t].flag) {
				DNchunk* c = &vol->chunks[vol->map[t].chunkIndex];
				dn_chunk_record* r = &p->recs[nrecs];
				uint32_t n = stage_record(vol, c, nrecs, nvw);
				uint32_t slot;
				if (!alloc_slot(p, n, &slot)) {
					dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to stage a chunk on the device");
					o->flags = DN_PEND_VALID | DN_PEND_EXISTS | (c->updated ? DN_PEND_UPDATED : 0);
				} else {
					r->pos[0] = c->pos.x; r->pos[1] = c->pos.y; r->pos[2] = c->pos.z;
					r->voxBase = p->slotBase[slot];
					c->numVoxelsGpu = n;
					o->flags = DN_PEND_VALID | DN_PEND_EXISTS | DN_PEND_STAGED | (c->updated ? DN_PEND_UPDATED : 0);
					o->slot = slot;
					o->recordIndex = nrecs;
					p->tileSlot[t] = slot;
					nrecs++;
					nvw += 2ull * n;
				}
				c->updated = false;
			}
		}
		p->dirtyList.n = 0;
	} else {
		/* DN_READ: the request filter still sees edited chunks as updated (voxel.c:1470) */
		for (size_t k = 0; k < nd; k++) {
			uint32_t t = p->dirtyList.v[k];
			if (vol->map[t].flag && vol->chunks[vol->map[t].chunkIndex].updated) {
				dn_tile_op* o = &p->ops[nops++];
				o->tile = t; o->flags = DN_PEND_UPDATED; o->slot = DN_SLOT_NONE; o->recordIndex = 0;
			}
		}
	}
	p->syncs++;
	if (p->residency == DN_RESIDENCY_LRU && !lru_pass(vol, op, &nops, &nrecs, &nvw)) return false;
	if (p->groupsStaged > vol->lightingRequestCap) DN_set_max_lighting_requests(vol, (size_t)p->groupsStaged * 2);

	spOut->op = (uint32_t)op;
	spOut->split = (uint32_t)lightingSplit;
	spOut->frameNum = vol->frameNum;
	*nopsOut = nops;
	*nrecsOut = nrecs;
	*nvwOut = nvw;
	return true;
}

/* after the device work of a sync was issued: slots replaced or removed by it are reusable by later
 * uploads (stream order) */
static void sync_done(DNvolume* vol)
{
	DNvolumePriv* p = priv(vol);
	for (size_t k = 0; k < p->deferredSlots.n; k++) free_slot(p, p->deferredSlots.v[k]);
	p->deferredSlots.n = 0;
	vol->numVoxelNodes = (size_t)p->stagedChunks;
}

void DN_sync_gpu(DNvolume* vol, DNmemOp op, int lightingSplit)
{
	/* DN_sync_gpu, voxel.c:719-786 */
	DNvolumePriv* p = priv(vol);
	if (!need_device(vol, "DN_sync_gpu")) return;
	dn_sync_params sp;
	uint32_t nops = 0, nrecs = 0;
	uint64_t nvw = 0;
	if (!sync_prepare(vol, op, lightingSplit, &sp, &nops, &nrecs, &nvw)) return;
	int rc = sync_issue(vol, &sp, nops, nrecs, nvw, 0);
	if (rc != DN_CUDA_OK)
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "device sync failed: %s", dn_cuda_last_error());
	sync_done(vol);
}

/* ------------------------------------------------------------- drawing */

void DN_set_view_projection_matrices(DNvolume* vol, float aspectRatio, float nearPlane, float farPlane, DNmat4* view, DNmat4* projection)
{
	/* voxel.c:788-810 */
	DNmat3 rotate = DN_mat4_top_left(DN_mat4_rotate_euler(vol->camOrient));
	DNvec3 camFront;
	float f = 1.0f / tanf(DN_deg_to_rad(vol->camFOV * 0.5f));
	if (aspectRatio < 1.0f)
		camFront = DN_mat3_mult_vec3(rotate, (DNvec3){{0.0f, 0.0f, aspectRatio / tanf(DN_deg_to_rad(vol->camFOV * 0.5f))}});
	else
		camFront = DN_mat3_mult_vec3(rotate, (DNvec3){{0.0f, 0.0f, f}});
	*view = DN_mat4_lookat(vol->camPos, DN_vec3_add(vol->camPos, camFront), (DNvec3){{0.0f, 1.0f, 0.0f}});
	*projection = DN_mat4_perspective(vol->camFOV, 1.0f / aspectRatio, nearPlane, farPlane);
}

void DN_draw_matrices(DNmat4 view, DNmat4 projection, DNmat4* invView, DNmat4* invCenteredView, DNmat4* invProjection)
{
	/* voxel.c:845-853 */
	DNmat4 centered = view;
	centered.m[3][0] = 0.0f; centered.m[3][1] = 0.0f; centered.m[3][2] = 0.0f;
	*invView = DN_mat4_inv(view);
	*invCenteredView = DN_mat4_inv(centered);
	*invProjection = DN_mat4_inv(projection);
}

/* the draw parameters DN_draw passes to the device (voxel.c:812-881) */
static void draw_prepare(DNvolume* vol, const DNimage* output, DNmat4 view, DNmat4 projection, dn_draw_params* dp)
{
	DNmat4 iv, icv, ip;
	DN_draw_matrices(view, projection, &iv, &icv, &ip);
	DNmat4 M = DN_mat4_mult(icv, ip);
	memset(dp, 0, sizeof(*dp));
	for (int r = 0; r < 3; r++)
		dp->origin[r] = iv.m[0][r] * 0.0f + iv.m[1][r] * 0.0f + iv.m[2][r] * 0.0f + iv.m[3][r] * 1.0f;
	memcpy(dp->dirMat, M.m, sizeof(dp->dirMat));
	dp->width = output->width;
	dp->height = output->height;
	dp->viewMode = vol->camViewMode;
	dp->truncate16 = vol->truncateDispatch;
	memcpy(dp->sunStrength, vol->sunStrength.v, 12);
	memcpy(dp->skyBot, vol->skyGradientBot.v, 12);
	memcpy(dp->skyTop, vol->skyGradientTop.v, 12);
	dp->emissiveStrength = vol->emissiveStrength;
	memcpy(dp->invProj, ip.m, sizeof(dp->invProj));
}

/* ---- raster textures: device buffers standing in for the GL textures of the raster pass ---- */

#define DN_MAX_TEXTURES 4096

typedef struct DNtextureSlot
{
	float* dev;
	uint32_t width, height;
	DNtextureFormat format;
} DNtextureSlot;

static DNtextureSlot g_textures[DN_MAX_TEXTURES];   /* handle h is slot h - 1; dev == NULL: free */
static pthread_mutex_t g_textureLock = PTHREAD_MUTEX_INITIALIZER;

static size_t texel_floats(DNtextureFormat f) { return f == DN_TEXTURE_RGBA32F ? 4 : 1; }

int DN_texture_create(uint32_t width, uint32_t height, DNtextureFormat format)
{
	if (width == 0 || height == 0 || (format != DN_TEXTURE_RGBA32F && format != DN_TEXTURE_DEPTH32F)) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_texture_create: invalid size or format");
		return -1;
	}
	float* dev = NULL;
	if (dn_cuda_malloc((void**)&dev, (size_t)width * height * texel_floats(format) * sizeof(float)) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate a texture: %s", dn_cuda_last_error());
		return -1;
	}
	pthread_mutex_lock(&g_textureLock);
	int h = -1;
	for (int i = 0; i < DN_MAX_TEXTURES; i++)
		if (!g_textures[i].dev) {
			g_textures[i].dev = dev; g_textures[i].width = width; g_textures[i].height = height;
			g_textures[i].format = format;
			h = i + 1;
			break;
		}
	pthread_mutex_unlock(&g_textureLock);
	if (h < 0) {
		dn_cuda_free(dev);
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_texture_create: all %d texture handles are in use", DN_MAX_TEXTURES);
	}
	return h;
}

/* copies slot h's description; false for a handle that names no texture */
static bool texture_get(int h, DNtextureSlot* out)
{
	if (h < 1 || h > DN_MAX_TEXTURES) return false;
	pthread_mutex_lock(&g_textureLock);
	*out = g_textures[h - 1];
	pthread_mutex_unlock(&g_textureLock);
	return out->dev != NULL;
}

void DN_texture_destroy(int texture)
{
	DNtextureSlot t;
	if (!texture_get(texture, &t)) return;
	pthread_mutex_lock(&g_textureLock);
	memset(&g_textures[texture - 1], 0, sizeof(DNtextureSlot));
	pthread_mutex_unlock(&g_textureLock);
	dn_cuda_free(t.dev);   /* waits for device work in flight */
}

bool DN_texture_upload(int texture, const float* texels)
{
	DNtextureSlot t;
	if (!texels || !texture_get(texture, &t)) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_texture_upload: invalid texture or data");
		return false;
	}
	if (dn_cuda_memcpy_h2d(t.dev, texels, (size_t)t.width * t.height * texel_floats(t.format) * sizeof(float)) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "texture upload failed: %s", dn_cuda_last_error());
		return false;
	}
	return true;
}

int DN_texture_format(int texture)
{
	DNtextureSlot t;
	return texture_get(texture, &t) ? (int)t.format : -1;
}

float* DN_texture_device_pointer(int texture, uint32_t* width, uint32_t* height)
{
	DNtextureSlot t;
	if (!texture_get(texture, &t)) return NULL;
	if (width) *width = t.width;
	if (height) *height = t.height;
	return t.dev;
}

/* raster composition of a draw: the reference composes when both handles are >= 0 (voxel.c:833-842); a
 * handle of 0 or below names no texture here (as GL never names a created texture 0).  False (with an
 * error message) when a positive handle names no texture of the right format. */
static bool raster_prepare(int colorTex, int depthTex, dn_draw_params* dp, const char* who)
{
	dp->compose = 0;
	if (colorTex <= 0 || depthTex <= 0) return true;
	DNtextureSlot c, d;
	if (!texture_get(colorTex, &c) || c.format != DN_TEXTURE_RGBA32F) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "%s: raster colour texture %d is not an RGBA32F texture", who, colorTex);
		return false;
	}
	if (!texture_get(depthTex, &d) || d.format != DN_TEXTURE_DEPTH32F) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "%s: raster depth texture %d is not a DEPTH32F texture", who, depthTex);
		return false;
	}
	dp->compose = 1;
	dp->rasterColor = c.dev; dp->rasterColorW = c.width; dp->rasterColorH = c.height;
	dp->rasterDepth = d.dev; dp->rasterDepthW = d.width; dp->rasterDepthH = d.height;
	return true;
}

void DN_draw(DNvolume* vol, DNimage* output, DNmat4 view, DNmat4 projection, int rasterColorTexture, int rasterDepthTexture)
{
	/* DN_draw, voxel.c:812-881 */
	if (!need_device(vol, "DN_draw")) return;
	if (!output || !output->color || output->width == 0 || output->height == 0) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "DN_draw: invalid output image");
		return;
	}
	if (vol->useCubemap)
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_NOTE, "cube-map sky is not available; using the sky gradient");
	dn_draw_params dp;
	draw_prepare(vol, output, view, projection, &dp);
	if (!raster_prepare(rasterColorTexture, rasterDepthTexture, &dp, "DN_draw")) return;
	int rc = output->onDevice
		? dn_cuda_draw(vol->gpu, &dp, (const dn_material*)vol->materials, output->color, output->hitIndex, output->hitFace)
		: dn_cuda_draw_host(vol->gpu, &dp, (const dn_material*)vol->materials, output->color, output->hitIndex, output->hitFace);
	if (rc != DN_CUDA_OK)
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "draw failed: %s", dn_cuda_last_error());
}

static void sphere_points(uint32_t K, float out[64][3])
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

/* the lighting parameters DN_update_lighting passes to the device (voxel.c:883-952); latches the time on
 * the first frame of a lighting split */
static void light_prepare(DNvolume* vol, int numDiffuseSamples, int maxDiffuseSamples, float time, dn_light_params* lpOut)
{
	DNvolumePriv* p = priv(vol);
	if (vol->frameNum == 0) vol->lastTime = time;
	dn_light_params lp;
	memset(&lp, 0, sizeof(lp));
	DNvec3 sd = DN_vec3_normalize(vol->sunDir);
	memcpy(lp.sunDir, sd.v, 12);
	memcpy(lp.sunStrength, vol->sunStrength.v, 12);
	memcpy(lp.ambient, vol->ambientLightStrength.v, 12);
	memcpy(lp.camPos, vol->camPos.v, 12);
	memcpy(lp.skyBot, vol->skyGradientBot.v, 12);
	memcpy(lp.skyTop, vol->skyGradientTop.v, 12);
	lp.shadowSoftness = vol->shadowSoftness;
	lp.time = vol->lastTime;
	lp.emissiveStrength = vol->emissiveStrength;
	lp.numDiffuse = numDiffuseSamples > 0 ? (uint32_t)numDiffuseSamples : 0u;
	lp.maxDiffuse = maxDiffuseSamples > 0 ? (uint32_t)maxDiffuseSamples : 0u;
	lp.diffuseBounceLimit = vol->diffuseBounceLimit;
	lp.specBounceLimit = vol->specBounceLimit;
	uint32_t K = vol->numDirectRays;
	if (K < 1) K = 1;
	if (K > 64) K = 64;
	lp.K = K;
	lp.rngMode = vol->rngMode;
	lp.mapId = vol->mapId;
	if (!p->sphereValid || p->sphereK != (float)K) {
		sphere_points(K, p->spherePts);
		p->sphereK = (float)K;
		p->sphereValid = 1;
	}
	memcpy(lp.spherePts, p->spherePts, sizeof(lp.spherePts));
	*lpOut = lp;
}

void DN_update_lighting(DNvolume* vol, int numDiffuseSamples, int maxDiffuseSamples, float time)
{
	/* DN_update_lighting, voxel.c:883-952 */
	if (!need_device(vol, "DN_update_lighting")) return;
	dn_light_params lp;
	light_prepare(vol, numDiffuseSamples, maxDiffuseSamples, time, &lp);
	int rc = dn_cuda_light(vol->gpu, &lp, (const dn_material*)vol->materials);
	if (rc != DN_CUDA_OK)
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "lighting update failed: %s", dn_cuda_last_error());
}

/* ----------------------------------------------------------- additions */

bool DN_finish(DNvolume* vol)
{
	if (!need_device(vol, "DN_finish")) return false;
	uint64_t nreq = 0;
	int rc = dn_cuda_finish(vol->gpu, &nreq);
	vol->numLightingRequests = (size_t)nreq;
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "device work failed: %s", dn_cuda_last_error());
		return false;
	}
	return true;
}

DNimage* DN_image_create(uint32_t width, uint32_t height, int onDevice, int withHitInfo)
{
	DNimage* img = (DNimage*)DN_MALLOC(sizeof(DNimage));
	if (!img) return NULL;
	memset(img, 0, sizeof(*img));
	img->width = width; img->height = height; img->onDevice = onDevice ? 1 : 0;
	size_t n = (size_t)width * height;
	int rc;
	if (onDevice) {
		rc = dn_cuda_malloc((void**)&img->color, n * 16);
		if (rc == DN_CUDA_OK && withHitInfo) rc = dn_cuda_malloc((void**)&img->hitIndex, n * 4);
		if (rc == DN_CUDA_OK && withHitInfo) rc = dn_cuda_malloc((void**)&img->hitFace, n);
	} else {
		rc = dn_cuda_malloc_host((void**)&img->color, n * 16);
		if (rc == DN_CUDA_OK && withHitInfo) rc = dn_cuda_malloc_host((void**)&img->hitIndex, n * 4);
		if (rc == DN_CUDA_OK && withHitInfo) rc = dn_cuda_malloc_host((void**)&img->hitFace, n);
	}
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate an image: %s", dn_cuda_last_error());
		DN_image_destroy(img);
		return NULL;
	}
	return img;
}

void DN_image_destroy(DNimage* img)
{
	if (!img) return;
	if (img->onDevice) { dn_cuda_free(img->color); dn_cuda_free(img->hitIndex); dn_cuda_free(img->hitFace); }
	else { dn_cuda_free_host(img->color); dn_cuda_free_host(img->hitIndex); dn_cuda_free_host(img->hitFace); }
	DN_FREE(img);
}

bool DN_get_stats(DNvolume* vol, DNstats* out)
{
	if (!need_device(vol, "DN_get_stats")) return false;
	dn_stats s;
	if (dn_cuda_stats(vol->gpu, &s) != DN_CUDA_OK) return false;
	out->rays = s.rays; out->primaryRays = s.primary; out->outerSteps = s.outerSteps;
	out->chunksEntered = s.chunksEntered; out->innerSteps = s.innerSteps; out->hits = s.hits;
	out->litVoxels = s.litVoxels; out->degenerate = s.degenerate;
	return true;
}

void DN_reset_stats(DNvolume* vol) { if (vol->gpu) dn_cuda_reset_stats(vol->gpu); }

size_t DN_export_lighting(DNvolume* vol, uint32_t* index, float* diffuse, float* specular, size_t capacity)
{
	uint64_t n = 0;
	if (!need_device(vol, "DN_export_lighting")) return 0;
	if (dn_cuda_export_lighting(vol->gpu, index, diffuse, specular, capacity, &n) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "lighting export failed: %s", dn_cuda_last_error());
		return 0;
	}
	return (size_t)n;
}

bool DN_export_tiles(DNvolume* vol, uint8_t* state, uint8_t* visible, uint32_t* lastUsed, uint32_t* samples)
{
	if (!need_device(vol, "DN_export_tiles")) return false;
	return dn_cuda_export_tiles(vol->gpu, state, visible, lastUsed, samples) == DN_CUDA_OK;
}

size_t DN_export_requests(DNvolume* vol, uint32_t* out, size_t capacity)
{
	uint64_t n = 0;
	if (!need_device(vol, "DN_export_requests")) return 0;
	if (dn_cuda_export_requests(vol->gpu, out, capacity, &n) != DN_CUDA_OK) return 0;
	return (size_t)n;
}

/* addition: struct sizes and field offsets, for language bindings that mirror these structs */
size_t DN_abi_layout(uint64_t* out, size_t n)
{
	const uint64_t v[] = {
		sizeof(DNvolume), offsetof(DNvolume, mapSize), offsetof(DNvolume, map), offsetof(DNvolume, chunks),
		offsetof(DNvolume, materials), offsetof(DNvolume, camPos), offsetof(DNvolume, sunDir),
		offsetof(DNvolume, useCubemap), offsetof(DNvolume, frameNum), offsetof(DNvolume, emissiveStrength),
		offsetof(DNvolume, deviceBudgetBytes), sizeof(DNchunk), sizeof(DNmaterial), sizeof(DNimage),
		sizeof(DNchunkHandle), sizeof(DNstats), offsetof(DNchunk, voxels), sizeof(DNvoxel),
		sizeof(DNbatchItem), offsetof(DNbatchItem, view), offsetof(DNbatchItem, op), offsetof(DNbatchItem, time),
		sizeof(DNrequest), offsetof(DNrequest, edits), offsetof(DNrequest, user), sizeof(DNcompletion),
		sizeof(DNvoxelEdit), sizeof(DNserveStats), offsetof(DNbatchItem, rasterColorTexture),
		offsetof(DNrequest, rasterColorTexture), sizeof(dn_draw_params), offsetof(dn_draw_params, compose),
		sizeof(dn_light_params)
	};
	size_t k = sizeof(v) / sizeof(v[0]);
	for (size_t i = 0; i < n && i < k; i++) out[i] = v[i];
	return k;
}

void DN_export_voxels(const DNvolume* vol, uint32_t* normalWords, uint32_t* albedoWords, uint8_t* tileFlags)
{
	const uint32_t X = vol->mapSize.x * DN_CHUNK_SIZE, Y = vol->mapSize.y * DN_CHUNK_SIZE;
	for (uint32_t tz = 0; tz < vol->mapSize.z; tz++)
	for (uint32_t ty = 0; ty < vol->mapSize.y; ty++)
	for (uint32_t tx = 0; tx < vol->mapSize.x; tx++) {
		const size_t t = tx + (size_t)vol->mapSize.x * (ty + (size_t)vol->mapSize.y * tz);
		const DNchunkHandle h = vol->map[t];
		if (tileFlags) tileFlags[t] = (uint8_t)h.flag;
		const DNchunk* c = h.flag ? &vol->chunks[h.chunkIndex] : NULL;
		for (uint32_t z = 0; z < DN_CHUNK_SIZE; z++)
		for (uint32_t y = 0; y < DN_CHUNK_SIZE; y++)
		for (uint32_t x = 0; x < DN_CHUNK_SIZE; x++) {
			const size_t v = (tx * 8 + x) + (size_t)X * ((ty * 8 + y) + (size_t)Y * (tz * 8 + z));
			const DNcompressedVoxel w = c ? c->voxels[x][y][z] : (DNcompressedVoxel){0xFFFFFFFFu, 0u};
			normalWords[v] = w.normal;
			albedoWords[v] = GET_MATERIAL_ID(w.normal) == DN_MATERIAL_EMPTY ? 0u : w.albedo;
		}
	}
}

/* addition: the chunk packing DN_sync_gpu applies to every changed chunk (voxel.c:1397-1461), exported
 * for tests and tools: mask[16], partial[3], 2 words per surface voxel; returns the voxel count */
uint32_t dn_pack_chunk(const DNvolume* vol, const DNchunk* chunk, uint32_t mask[16], uint32_t partial[3], uint32_t* words)
{
	static int tableReady = 0;
	if (!tableReady) { init_linear_table(); tableReady = 1; }
	dn_chunk_record r;
	uint32_t n = pack_chunk(vol, chunk, &r, words);
	memcpy(mask, r.mask, sizeof(r.mask));
	memcpy(partial, r.partial, sizeof(r.partial));
	return n;
}

uint32_t dn_count_surface(const DNvolume* vol, const DNchunk* chunk)
{
	dn_pack_params pk;
	pack_params(vol, &pk);
	return count_kept(chunk, pk.seeThrough);
}

/* ---------------------------------------------------------------- batches */

struct DNbatch
{
	struct DNgpuBatch* gpu;
	DNvolume** members; size_t nmembers, membersCap;
	dn_batch_item* items; size_t itemsCap;
	uint64_t runs;
};

DNbatch* DN_batch_create(void)
{
	DNbatch* b = (DNbatch*)DN_MALLOC(sizeof(DNbatch));
	if (!b) { dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate a batch"); return NULL; }
	memset(b, 0, sizeof(*b));
	if (dn_cuda_batch_create(&b->gpu) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "failed to create a batch: %s", dn_cuda_last_error());
		DN_FREE(b);
		return NULL;
	}
	return b;
}

void DN_batch_destroy(DNbatch* b)
{
	if (!b) return;
	for (size_t i = 0; i < b->nmembers; i++) priv(b->members[i])->batch = NULL;
	dn_cuda_batch_destroy(b->gpu);
	DN_FREE(b->members);
	DN_FREE(b->items);
	DN_FREE(b);
}

bool DN_batch_add(DNbatch* b, DNvolume* vol)
{
	if (!b || !vol || !need_device(vol, "DN_batch_add")) return false;
	if (priv(vol)->batch) { dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_batch_add: the volume already belongs to a batch"); return false; }
	if (priv(vol)->residency != DN_RESIDENCY_KEEP) { dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_batch_add: batches hold DN_RESIDENCY_KEEP volumes only"); return false; }
	if (!grow_scratch((void**)&b->members, &b->membersCap, b->nmembers + 1, sizeof(DNvolume*))) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to grow a batch");
		return false;
	}
	if (dn_cuda_batch_add(b->gpu, vol->gpu) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_batch_add: %s", dn_cuda_last_error());
		return false;
	}
	b->members[b->nmembers++] = vol;
	priv(vol)->batch = b;
	return true;
}

bool DN_batch_remove(DNbatch* b, DNvolume* vol)
{
	if (!b || !vol || priv(vol)->batch != b) return false;
	for (size_t i = 0; i < b->nmembers; i++) {
		if (b->members[i] != vol) continue;
		b->members[i] = b->members[--b->nmembers];
		priv(vol)->batch = NULL;
		if (dn_cuda_batch_remove(b->gpu, vol->gpu) != DN_CUDA_OK) {
			dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_batch_remove: %s", dn_cuda_last_error());
			return false;
		}
		return true;
	}
	return false;
}

bool DN_batch_run(DNbatch* b, const DNbatchItem* items, unsigned int count)
{
	if (!b || (!items && count)) return false;
	if (!grow_scratch((void**)&b->items, &b->itemsCap, count ? count : 1, sizeof(dn_batch_item))) {
		dn_msg(DN_MESSAGE_CPU_MEMORY, DN_MESSAGE_ERROR, "failed to allocate batch items");
		return false;
	}
	/* every item is checked before any volume's state moves */
	const uint64_t run = ++b->runs;
	for (unsigned int i = 0; i < count; i++) {
		const DNbatchItem* it = &items[i];
		DNvolume* vol = it->vol;
		if (!vol || priv(vol)->batch != b) {
			dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_batch_run: item %u is not a member of the batch", i);
			return false;
		}
		if (priv(vol)->batchStamp == run) {
			dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "DN_batch_run: item %u repeats a volume of this run", i);
			return false;
		}
		priv(vol)->batchStamp = run;
		const DNimage* out = it->output;
		if ((it->phases & DN_PHASE_DRAW) && (!out || !out->color || out->width == 0 || out->height == 0)) {
			dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "DN_batch_run: item %u has an invalid output image", i);
			return false;
		}
		dn_draw_params probe;
		if ((it->phases & DN_PHASE_DRAW) && !raster_prepare(it->rasterColorTexture, it->rasterDepthTexture, &probe, "DN_batch_run"))
			return false;
	}
	/* host halves in item order: draw parameters, chunk staging (issued now on the batch's stream; the
	 * staged records are published by the sync pass, after the draw), lighting parameters */
	for (unsigned int i = 0; i < count; i++) {
		const DNbatchItem* it = &items[i];
		DNvolume* vol = it->vol;
		dn_batch_item* d = &b->items[i];
		memset(d, 0, sizeof(*d));
		d->map = vol->gpu;
		d->phases = it->phases & (DN_PHASE_DRAW | DN_PHASE_SYNC | DN_PHASE_LIGHT);
		d->materials = (const dn_material*)vol->materials;
		if (it->phases & DN_PHASE_DRAW) {
			const DNimage* out = it->output;
			draw_prepare(vol, out, it->view, it->projection, &d->draw);
			if (!raster_prepare(it->rasterColorTexture, it->rasterDepthTexture, &d->draw, "DN_batch_run")) return false;
			d->hostImage = out->onDevice ? 0u : 1u;
			d->colorOut = out->color; d->hitOut = out->hitIndex; d->faceOut = out->hitFace;
		}
		if (it->phases & DN_PHASE_SYNC) {
			DNvolumePriv* p = priv(vol);
			uint32_t nops = 0, nrecs = 0;
			uint64_t nvw = 0;
			if (!sync_prepare(vol, it->op, it->lightingSplit, &d->sync, &nops, &nrecs, &nvw)) return false;
			int rc = sync_issue(vol, NULL, nops, nrecs, nvw, 1);
			sync_done(vol);
			if (rc != DN_CUDA_OK) {
				dn_msg(DN_MESSAGE_GPU_MEMORY, DN_MESSAGE_ERROR, "device sync failed: %s", dn_cuda_last_error());
				return false;
			}
		}
		if (it->phases & DN_PHASE_LIGHT) light_prepare(vol, it->numDiffuseSamples, it->maxDiffuseSamples, it->time, &d->light);
	}
	if (dn_cuda_batch_frame(b->gpu, b->items, count) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "batched frame failed: %s", dn_cuda_last_error());
		return false;
	}
	return true;
}

bool DN_batch_finish(DNbatch* b)
{
	if (!b) return false;
	int rc = dn_cuda_batch_finish(b->gpu);
	for (size_t i = 0; i < b->nmembers; i++)
		b->members[i]->numLightingRequests = (size_t)dn_cuda_requests_of(b->members[i]->gpu);
	if (rc != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "batched device work failed: %s", dn_cuda_last_error());
		return false;
	}
	return true;
}

bool DN_batch_get_stats(DNbatch* b, DNstats* out)
{
	dn_stats s;
	if (!b || !out || dn_cuda_batch_stats(b->gpu, 0, &s) != DN_CUDA_OK) return false;
	out->rays = s.rays; out->primaryRays = s.primary; out->outerSteps = s.outerSteps;
	out->chunksEntered = s.chunksEntered; out->innerSteps = s.innerSteps; out->hits = s.hits;
	out->litVoxels = s.litVoxels; out->degenerate = s.degenerate;
	return true;
}

void DN_batch_reset_stats(DNbatch* b) { if (b) dn_cuda_batch_reset_stats(b->gpu); }

bool DN_batch_autotune(DNbatch* b)
{
	if (!b) return false;
	if (dn_cuda_batch_autotune(b->gpu, NULL) != DN_CUDA_OK) {
		dn_msg(DN_MESSAGE_SHADER, DN_MESSAGE_ERROR, "batch autotuning failed: %s", dn_cuda_last_error());
		return false;
	}
	return true;
}

void* DN_batch_stream(DNbatch* b) { return b ? dn_cuda_batch_stream(b->gpu) : NULL; }
