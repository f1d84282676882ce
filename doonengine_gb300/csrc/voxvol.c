/*
 * voxvol.c -- the .voxvol volume file format (DN_load_volume / DN_save_volume).
 *
 * Byte layout, identical to the reference (src/DoonEngine/voxel.c:520-654):
 *   DNuvec3 mapSize | size_t chunkCap | chunkCap x (uint16 size, compressed chunk)
 *   | DNmaterial[256] | camPos, camOrient (DNvec3), camFOV (float), camViewMode (u32)
 *   | sunDir, sunStrength, ambientLightStrength (DNvec3), diffuseBounceLimit,
 *     specBounceLimit (u32), shadowSoftness (float) | skyGradientBot, skyGradientTop
 * Compressed chunk (voxel.c:301-518): DNivec3 pos; if pos is outside the map
 * nothing else.  Otherwise a normal palette and an albedo palette (u8 count +
 * 3 bytes per entry; a palette is used only while it stays below
 * numVoxels/2 entries, else its count is 0), then runs over the voxels in
 * x-fastest order: u8 material, u8 run length (<= 255), and for every
 * non-empty voxel of the run its normal (palette index or 3 bytes) and albedo
 * (palette index or 3 bytes).
 * Unlike the reference, loading checks every read and rejects truncated or
 * malformed files (zero-length runs, palette indices past the palette).
 */
#include "DoonEngine/voxel.h"
#include <string.h>

void DN_volume_mark_loaded_chunk(DNvolume* vol, size_t tile);   /* voxel.c */

typedef struct b3 { uint8_t x, y, z; } b3;

static int pal_find(const b3* p, int n, b3 v)
{
	for (int i = 0; i < n; i++)
		if (p[i].x == v.x && p[i].y == v.y && p[i].z == v.z) return i;
	return -1;
}

static void msg(DNmessageSeverity s, const char* m)
{
	if (g_DN_message_callback) g_DN_message_callback(DN_MESSAGE_FILE_IO, s, m);
}

/* returns the compressed size in bytes (mem must hold 2 * sizeof(DNchunk)) */
size_t DN_compress_chunk(const DNvolume* vol, const DNchunk* c, uint8_t* mem)
{
	uint8_t* p = mem;
	memcpy(p, &c->pos, sizeof(DNivec3)); p += sizeof(DNivec3);
	if (!DN_in_map_bounds((DNvolume*)vol, c->pos)) return (size_t)(p - mem);
	b3 np[DN_CHUNK_LENGTH / 2], ap[DN_CHUNK_LENGTH / 2];
	int nn = 0, na = 0;
	const int limit = (int)(c->numVoxels / 2);
	for (int z = 0; z < 8; z++)
	for (int y = 0; y < 8; y++)
	for (int x = 0; x < 8; x++) {
		uint32_t nw = c->voxels[x][y][z].normal, aw = c->voxels[x][y][z].albedo;
		if ((nw >> 24) == DN_MATERIAL_EMPTY) continue;
		b3 n = {(uint8_t)(nw >> 16), (uint8_t)(nw >> 8), (uint8_t)nw};
		b3 a = {(uint8_t)(aw >> 24), (uint8_t)(aw >> 16), (uint8_t)(aw >> 8)};
		if (nn < limit && pal_find(np, nn, n) < 0) np[nn++] = n;
		if (na < limit && pal_find(ap, na, a) < 0) ap[na++] = a;
	}
	if (!(nn < limit)) nn = 0;
	if (!(na < limit)) na = 0;
	*p++ = (uint8_t)nn; memcpy(p, np, 3 * (size_t)nn); p += 3 * (size_t)nn;
	*p++ = (uint8_t)na; memcpy(p, ap, 3 * (size_t)na); p += 3 * (size_t)na;
	for (int i = 0; i < DN_CHUNK_LENGTH; ) {
		int x = i % 8, y = (i / 8) % 8, z = i / 64;
		uint8_t mat = (uint8_t)(c->voxels[x][y][z].normal >> 24);
		*p++ = mat;
		uint8_t* countAt = p++;
		uint8_t num = 0;
		int j = i;
		for (; j < DN_CHUNK_LENGTH; j++) {
			int x2 = j % 8, y2 = (j / 8) % 8, z2 = j / 64;
			uint32_t nw = c->voxels[x2][y2][z2].normal, aw = c->voxels[x2][y2][z2].albedo;
			if (num >= 255 || (uint8_t)(nw >> 24) != mat) break;
			num++;
			if (mat == DN_MATERIAL_EMPTY) continue;
			b3 n = {(uint8_t)(nw >> 16), (uint8_t)(nw >> 8), (uint8_t)nw};
			b3 a = {(uint8_t)(aw >> 24), (uint8_t)(aw >> 16), (uint8_t)(aw >> 8)};
			if (nn > 0) *p++ = (uint8_t)pal_find(np, nn, n);
			else { memcpy(p, &n, 3); p += 3; }
			if (na > 0) *p++ = (uint8_t)pal_find(ap, na, a);
			else { memcpy(p, &a, 3); p += 3; }
		}
		*countAt = num;
		i = j;
	}
	return (size_t)(p - mem);
}

/* returns 0 on success; the chunk is cleared first */
int DN_decompress_chunk(const DNvolume* vol, const uint8_t* mem, size_t size, DNchunk* c)
{
	const uint8_t* p = mem;
	const uint8_t* end = mem + size;
#define NEED(k) do { if ((size_t)(end - p) < (size_t)(k)) return -1; } while (0)
	NEED(sizeof(DNivec3));
	memcpy(&c->pos, p, sizeof(DNivec3)); p += sizeof(DNivec3);
	c->updated = false;
	c->numVoxels = 0;
	c->numVoxelsGpu = 0;
	for (int x = 0; x < 8; x++) for (int y = 0; y < 8; y++) for (int z = 0; z < 8; z++) c->voxels[x][y][z].normal = UINT32_MAX;
	if (!DN_in_map_bounds((DNvolume*)vol, c->pos)) return 0;
	b3 np[256], ap[256];
	NEED(1); uint8_t nn = *p++;
	NEED(3 * (size_t)nn); memcpy(np, p, 3 * (size_t)nn); p += 3 * (size_t)nn;
	NEED(1); uint8_t na = *p++;
	NEED(3 * (size_t)na); memcpy(ap, p, 3 * (size_t)na); p += 3 * (size_t)na;
	int read = 0;
	while (read < DN_CHUNK_LENGTH) {
		NEED(2);
		uint8_t mat = *p++, num = *p++;
		if (num == 0 || read + num > DN_CHUNK_LENGTH) return -1;
		for (int i = read; i < read + num; i++) {
			int x = i % 8, y = (i / 8) % 8, z = i / 64;
			if (mat == DN_MATERIAL_EMPTY) { c->voxels[x][y][z].normal = UINT32_MAX; continue; }
			b3 n, a;
			if (nn > 0) { NEED(1); uint8_t k = *p++; if (k >= nn) return -1; n = np[k]; }
			else { NEED(3); memcpy(&n, p, 3); p += 3; }
			if (na > 0) { NEED(1); uint8_t k = *p++; if (k >= na) return -1; a = ap[k]; }
			else { NEED(3); memcpy(&a, p, 3); p += 3; }
			c->voxels[x][y][z].normal = ((uint32_t)mat << 24) | ((uint32_t)n.x << 16) | ((uint32_t)n.y << 8) | n.z;
			c->voxels[x][y][z].albedo = ((uint32_t)a.x << 24) | ((uint32_t)a.y << 16) | ((uint32_t)a.z << 8);
			c->numVoxels++;
		}
		read += num;
	}
#undef NEED
	return 0;
}

static int rd(FILE* f, void* d, size_t n) { return fread(d, 1, n, f) == n; }

DNvolume* DN_load_volume(const char* filePath, unsigned int minChunks)
{
	FILE* f = fopen(filePath, "rb");
	if (!f) {
		char m[512];
		snprintf(m, sizeof(m), "failed to open file \"%s\" for reading", filePath);
		msg(DN_MESSAGE_ERROR, m);
		return NULL;
	}
	DNuvec3 mapSize;
	uint64_t chunkCap = 0;
	DNvolume* vol = NULL;
	uint8_t* buf = NULL;
	if (!rd(f, &mapSize, sizeof(mapSize)) || !rd(f, &chunkCap, sizeof(chunkCap))) goto bad;
	if ((uint64_t)mapSize.x * mapSize.y * mapSize.z == 0 || chunkCap == 0 ||
	    chunkCap > (uint64_t)mapSize.x * mapSize.y * mapSize.z + 1024u) goto bad;
	vol = DN_create_volume(mapSize, minChunks);
	if (!vol) { fclose(f); return NULL; }
	if (!DN_set_max_chunks(vol, (size_t)chunkCap)) goto fail;
	buf = (uint8_t*)DN_MALLOC(65536);
	if (!buf) goto fail;
	for (uint64_t i = 0; i < chunkCap; i++) {
		uint16_t sz;
		if (!rd(f, &sz, 2) || !rd(f, buf, sz)) goto bad;
		if (DN_decompress_chunk(vol, buf, sz, &vol->chunks[i]) != 0) goto bad;
		if (DN_in_map_bounds(vol, vol->chunks[i].pos)) {
			size_t t = DN_FLATTEN_INDEX(vol->chunks[i].pos, mapSize);
			vol->map[t].flag = 1;
			vol->map[t].chunkIndex = (uint32_t)i;
			DN_volume_mark_loaded_chunk(vol, t);
		}
	}
	if (!rd(f, vol->materials, sizeof(DNmaterial) * DN_MAX_MATERIALS)) goto bad;
	if (!rd(f, &vol->camPos, 12) || !rd(f, &vol->camOrient, 12) || !rd(f, &vol->camFOV, 4) || !rd(f, &vol->camViewMode, 4)) goto bad;
	if (!rd(f, &vol->sunDir, 12) || !rd(f, &vol->sunStrength, 12) || !rd(f, &vol->ambientLightStrength, 12) ||
	    !rd(f, &vol->diffuseBounceLimit, 4) || !rd(f, &vol->specBounceLimit, 4) || !rd(f, &vol->shadowSoftness, 4)) goto bad;
	if (!rd(f, &vol->skyGradientBot, 12) || !rd(f, &vol->skyGradientTop, 12)) goto bad;
	DN_FREE(buf);
	fclose(f);
	return vol;
bad:
	msg(DN_MESSAGE_ERROR, "malformed or truncated volume file");
fail:
	DN_FREE(buf);
	if (vol) DN_delete_volume(vol);
	fclose(f);
	return NULL;
}

bool DN_save_volume(const char* filePath, DNvolume* vol)
{
	FILE* f = fopen(filePath, "wb");
	if (!f) {
		char m[512];
		snprintf(m, sizeof(m), "failed to open file \"%s\" for writing", filePath);
		msg(DN_MESSAGE_ERROR, m);
		return false;
	}
	uint8_t* buf = (uint8_t*)DN_MALLOC(sizeof(DNchunk) * 2);
	if (!buf) { fclose(f); return false; }
	uint64_t cap = vol->chunkCap;
	int ok = fwrite(&vol->mapSize, sizeof(DNuvec3), 1, f) == 1 && fwrite(&cap, 8, 1, f) == 1;
	for (size_t i = 0; ok && i < vol->chunkCap; i++) {
		size_t n = DN_compress_chunk(vol, &vol->chunks[i], buf);
		uint16_t s16 = (uint16_t)n;
		ok = n <= 65535 && fwrite(&s16, 2, 1, f) == 1 && fwrite(buf, 1, n, f) == n;
	}
	ok = ok && fwrite(vol->materials, sizeof(DNmaterial), DN_MAX_MATERIALS, f) == DN_MAX_MATERIALS;
	ok = ok && fwrite(&vol->camPos, 12, 1, f) == 1 && fwrite(&vol->camOrient, 12, 1, f) == 1 &&
	     fwrite(&vol->camFOV, 4, 1, f) == 1 && fwrite(&vol->camViewMode, 4, 1, f) == 1;
	ok = ok && fwrite(&vol->sunDir, 12, 1, f) == 1 && fwrite(&vol->sunStrength, 12, 1, f) == 1 &&
	     fwrite(&vol->ambientLightStrength, 12, 1, f) == 1 && fwrite(&vol->diffuseBounceLimit, 4, 1, f) == 1 &&
	     fwrite(&vol->specBounceLimit, 4, 1, f) == 1 && fwrite(&vol->shadowSoftness, 4, 1, f) == 1;
	ok = ok && fwrite(&vol->skyGradientBot, 12, 1, f) == 1 && fwrite(&vol->skyGradientTop, 12, 1, f) == 1;
	DN_FREE(buf);
	fclose(f);
	if (!ok) msg(DN_MESSAGE_ERROR, "failed to write the volume file");
	return ok != 0;
}
