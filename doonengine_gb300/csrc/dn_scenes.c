/*
 * dn_scenes.c -- seeded synthetic maps for benchmarks and tests (addition;
 * the reference ships only a demo scene).  Everything goes through the
 * public edit API (DN_set_compressed_voxel), so a generated map is an
 * ordinary DNvolume.
 *
 *   dn_scene_palette   16-style material palette: linear albedo U[lo,hi]^3,
 *                      specular U[0,specMax], nEmissive emissive materials
 *   dn_scene_terrain   value-noise heightfield (3 octaves), solid below the
 *                      surface, normals from the height gradient
 *   dn_scene_shapes    seeded boxes and spheres
 *   dn_scene_camera    a camera above the terrain looking across it
 *   dn_scene_reroll    re-rolls the voxels of chosen chunks (streaming edits)
 * Per-voxel albedo bytes are the sRGB encoding of the material's linear
 * albedo (x^(1/2.2)), so the reference's upload-time linearisation
 * (voxel.c:1441-1447) gives back approximately the palette value.
 */
#include "DoonEngine/voxel.h"
#include <math.h>
#include <string.h>

typedef struct rng { uint64_t s; } rng;
static uint32_t rnext(rng* r)
{
	/* splitmix64 */
	uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return (uint32_t)((z ^ (z >> 31)) >> 32);
}
static float runif(rng* r) { return (float)(rnext(r) >> 8) * (1.0f / 16777216.0f); }

static uint32_t lattice(uint32_t seed, int32_t x, int32_t z)
{
	uint32_t h = seed ^ ((uint32_t)x * 0x8da6b343u) ^ ((uint32_t)z * 0xd8163841u);
	h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
	return h;
}

static float value_noise(uint32_t seed, float x, float z)
{
	int32_t ix = (int32_t)floorf(x), iz = (int32_t)floorf(z);
	float fx = x - (float)ix, fz = z - (float)iz;
	float sx = fx * fx * (3.0f - 2.0f * fx), sz = fz * fz * (3.0f - 2.0f * fz);
	float a = (float)(lattice(seed, ix, iz) >> 8) / 16777216.0f;
	float b = (float)(lattice(seed, ix + 1, iz) >> 8) / 16777216.0f;
	float c = (float)(lattice(seed, ix, iz + 1) >> 8) / 16777216.0f;
	float d = (float)(lattice(seed, ix + 1, iz + 1) >> 8) / 16777216.0f;
	float ab = a + (b - a) * sx, cd = c + (d - c) * sx;
	return ab + (cd - ab) * sz;
}

static float height_at(uint32_t seed, float x, float z, float base, float amp, float scale)
{
	float h = 0.0f, f = 1.0f / scale, w = 1.0f, tw = 0.0f;
	for (int o = 0; o < 3; o++) {
		h += w * value_noise(seed + (uint32_t)o * 101u, x * f, z * f);
		tw += w;
		w *= 0.5f; f *= 2.0f;
	}
	return base + amp * (h / tw - 0.5f) * 2.0f;
}

static uint8_t srgb_byte(float lin)
{
	float v = powf(lin < 0.0f ? 0.0f : (lin > 1.0f ? 1.0f : lin), 1.0f / 2.2f) * 255.0f + 0.5f;
	return (uint8_t)(v > 255.0f ? 255.0f : v);
}

static uint8_t s_palette[256][3];

void dn_scene_palette(DNvolume* vol, uint32_t seed, uint32_t nMaterials, uint32_t nEmissive,
                      float albedoLo, float albedoHi, float specMax)
{
	rng r = {((uint64_t)seed << 32) ^ 0xA5A5F00Dull};
	if (nMaterials > 255) nMaterials = 255;
	for (uint32_t m = 0; m < nMaterials; m++) {
		DNmaterial* mt = &vol->materials[m];
		memset(mt, 0, sizeof(*mt));
		for (int k = 0; k < 3; k++) s_palette[m][k] = srgb_byte(albedoLo + (albedoHi - albedoLo) * runif(&r));
		mt->opacity = 1.0f;
		mt->refractIndex = 1.0f;
		mt->specular = specMax * runif(&r);
		mt->reflectType = rnext(&r) & 1u;
		mt->shininess = 1u + rnext(&r) % 8u;
		mt->emissive = (m >= nMaterials - nEmissive) ? 1u : 0u;
		if (mt->emissive) mt->specular = 0.0f;
	}
}

static void put(DNvolume* vol, int32_t x, int32_t y, int32_t z, uint8_t mat, float nx, float ny, float nz)
{
	if (x < 0 || y < 0 || z < 0) return;
	if ((uint32_t)x >= vol->mapSize.x * 8u || (uint32_t)y >= vol->mapSize.y * 8u || (uint32_t)z >= vol->mapSize.z * 8u) return;
	DNvoxel v;
	v.material = mat;
	float l = sqrtf(nx * nx + ny * ny + nz * nz);
	if (l > 0.0f) { nx /= l; ny /= l; nz /= l; } else { ny = 1.0f; }
	v.normal.x = nx; v.normal.y = ny; v.normal.z = nz;
	v.albedo.r = s_palette[mat][0]; v.albedo.g = s_palette[mat][1]; v.albedo.b = s_palette[mat][2];
	DN_set_voxel(vol, (DNivec3){x / 8, y / 8, z / 8}, (DNivec3){x % 8, y % 8, z % 8}, v);
}

/* terrain: mean surface height meanFrac * (map height in voxels), amplitude ampFrac of it */
void dn_scene_terrain(DNvolume* vol, uint32_t seed, float meanFrac, float ampFrac, uint32_t nMaterials, uint32_t nEmissive)
{
	const int32_t X = (int32_t)vol->mapSize.x * 8, Y = (int32_t)vol->mapSize.y * 8, Z = (int32_t)vol->mapSize.z * 8;
	const float base = meanFrac * (float)Y, amp = ampFrac * (float)Y;
	const float scale = (float)(X > Z ? X : Z) / 6.0f + 8.0f;
	uint32_t nSolid = nMaterials > nEmissive ? nMaterials - nEmissive : 1;
	rng r = {((uint64_t)seed << 32) ^ 0x7E44A1Bull};
	for (int32_t z = 0; z < Z; z++)
	for (int32_t x = 0; x < X; x++) {
		float h = height_at(seed, (float)x, (float)z, base, amp, scale);
		float hx = height_at(seed, (float)x + 1.0f, (float)z, base, amp, scale) - height_at(seed, (float)x - 1.0f, (float)z, base, amp, scale);
		float hz = height_at(seed, (float)x, (float)z + 1.0f, base, amp, scale) - height_at(seed, (float)x, (float)z - 1.0f, base, amp, scale);
		int32_t top = (int32_t)h;
		if (top < 1) top = 1;
		if (top > Y) top = Y;
		float bandf = value_noise(seed ^ 0x5151u, (float)x / 24.0f, (float)z / 24.0f);
		uint8_t mat = (uint8_t)((uint32_t)(bandf * (float)nSolid) % nSolid);
		for (int32_t y = 0; y < top; y++) {
			uint8_t m = (y < top - 3) ? (uint8_t)((mat + 1u) % nSolid) : mat;
			put(vol, x, y, z, m, -hx * 0.5f, 1.0f, -hz * 0.5f);
		}
		/* sparse emissive "lamps" on the surface */
		if (nEmissive && (rnext(&r) % 4096u) == 0u)
			put(vol, x, top, z, (uint8_t)(nSolid + rnext(&r) % nEmissive), 0.0f, 1.0f, 0.0f);
	}
}

void dn_scene_shapes(DNvolume* vol, uint32_t seed, uint32_t nShapes, int32_t minSize, int32_t maxSize,
                     uint32_t nMaterials, float yLo, float yHi)
{
	const int32_t X = (int32_t)vol->mapSize.x * 8, Y = (int32_t)vol->mapSize.y * 8, Z = (int32_t)vol->mapSize.z * 8;
	rng r = {((uint64_t)seed << 32) ^ 0x5EEDB0Bull};
	for (uint32_t s = 0; s < nShapes; s++) {
		int32_t cx = (int32_t)(runif(&r) * (float)X), cz = (int32_t)(runif(&r) * (float)Z);
		int32_t cy = (int32_t)((yLo + (yHi - yLo) * runif(&r)) * (float)Y);
		int32_t size = minSize + (int32_t)(rnext(&r) % (uint32_t)(maxSize - minSize + 1));
		uint8_t mat = (uint8_t)(rnext(&r) % nMaterials);
		int sphere = rnext(&r) & 1u;
		int32_t hs = size / 2;
		for (int32_t dz = -hs; dz <= hs; dz++)
		for (int32_t dy = -hs; dy <= hs; dy++)
		for (int32_t dx = -hs; dx <= hs; dx++) {
			if (sphere) {
				if (dx * dx + dy * dy + dz * dz > hs * hs) continue;
				put(vol, cx + dx, cy + dy, cz + dz, mat, (float)dx, (float)dy, (float)dz);
			} else {
				int32_t ax = dx < 0 ? -dx : dx, ay = dy < 0 ? -dy : dy, az = dz < 0 ? -dz : dz;
				float nx = 0.0f, ny = 0.0f, nz = 0.0f;
				if (ax >= ay && ax >= az) nx = (float)dx; else if (ay >= az) ny = (float)dy; else nz = (float)dz;
				put(vol, cx + dx, cy + dy, cz + dz, mat, nx, ny, nz);
			}
		}
	}
}

/* camera in chunk units: from (fx, fy, fz) of the map extent, with pitch / yaw in degrees */
void dn_scene_camera(DNvolume* vol, float fx, float fy, float fz, float pitch, float yaw, float fov)
{
	vol->camPos.x = fx * (float)vol->mapSize.x;
	vol->camPos.y = fy * (float)vol->mapSize.y;
	vol->camPos.z = fz * (float)vol->mapSize.z;
	vol->camOrient.x = pitch;
	vol->camOrient.y = yaw;
	vol->camOrient.z = 0.0f;
	vol->camFOV = fov;
}

/* streaming edits: re-rolls the voxels of n existing chunks (pos: 3 ints per chunk, chunk units) from
 * seed -- each solid voxel takes a new solid material or (1 in 8) is removed, each empty voxel becomes
 * solid with probability 1/32 -- through the public edit API, so every chunk touched is marked for
 * re-upload at the next DN_sync_gpu */
void dn_scene_reroll(DNvolume* vol, const int32_t* pos, uint32_t n, uint32_t seed, uint32_t nMaterials)
{
	if (nMaterials == 0) nMaterials = 1;
	for (uint32_t c = 0; c < n; c++) {
		DNivec3 mp = {pos[3 * c], pos[3 * c + 1], pos[3 * c + 2]};
		if (!DN_in_map_bounds(vol, mp)) continue;
		rng r = {((uint64_t)seed << 32) ^ ((uint64_t)c * 0x9E3779B97F4A7C15ull) ^ 0xC4A7ull};
		for (int32_t z = 0; z < 8; z++)
		for (int32_t y = 0; y < 8; y++)
		for (int32_t x = 0; x < 8; x++) {
			DNivec3 cp = {x, y, z};
			const uint32_t u = rnext(&r);
			if (DN_does_voxel_exist(vol, mp, cp)) {
				if ((u & 7u) == 0u) { DN_remove_voxel(vol, mp, cp); continue; }
				DNvoxel v = DN_get_voxel(vol, mp, cp);
				v.material = (uint8_t)((u >> 8) % nMaterials);
				v.albedo.r = s_palette[v.material][0]; v.albedo.g = s_palette[v.material][1]; v.albedo.b = s_palette[v.material][2];
				DN_set_voxel(vol, mp, cp, v);
			} else if ((u & 31u) == 0u) {
				put(vol, mp.x * 8 + x, mp.y * 8 + y, mp.z * 8 + z, (uint8_t)((u >> 8) % nMaterials), 0.0f, 1.0f, 0.0f);
			}
		}
	}
}
