/*
 * voxelShapes.c -- the shape functions of include/DoonEngine/voxelShapes.h (the reference's
 * src/DoonEngine/voxelShapes.c:93-442).
 *
 * Host half of each shape: the transform and its inverse, the bounding box and the chunk range it covers
 * (the reference's rules, its quirks included), then dn_cuda_shape_eval for the per-voxel distances and
 * normals on the GPU, then the edits applied to the CPU map in the reference's visiting order (chunks
 * z, y, x; voxels z, y, x) with its rules (voxelShapes.c:191-231 and 288-331).
 */
#include "DoonEngine/voxelShapes.h"
#include "dn_cuda.h"
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern void (*g_DN_message_callback)(DNmessageType, DNmessageSeverity, const char*);

static void shape_msg(DNmessageSeverity s, const char* fmt, ...)
{
	char m[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(m, sizeof(m), fmt, ap);
	va_end(ap);
	if (g_DN_message_callback) g_DN_message_callback(DN_MESSAGE_CPU_MEMORY, s, m);
}

/* the transformed bounding box: the 8 corners through t, then their component-wise extremes
 * (voxelShapes.c:93-130) */
static void transform_bounds(DNvec3* min, DNvec3* max, DNmat4 t)
{
	const DNvec3 lo = *min, hi = *max;
	const DNvec3 pts[8] = {
		{{lo.x, lo.y, lo.z}}, {{lo.x, lo.y, hi.z}}, {{lo.x, hi.y, lo.z}}, {{lo.x, hi.y, hi.z}},
		{{hi.x, lo.y, lo.z}}, {{hi.x, lo.y, hi.z}}, {{hi.x, hi.y, lo.z}}, {{hi.x, hi.y, hi.z}}};
	DNvec3 mn = {{INFINITY, INFINITY, INFINITY}}, mx = {{-INFINITY, -INFINITY, -INFINITY}};
	for (int i = 0; i < 8; i++) {
		DNvec4 v = {{pts[i].x, pts[i].y, pts[i].z, 1.0f}};
		v = DN_mat4_mult_vec4(t, v);
		for (int k = 0; k < 3; k++) {
			if (v.v[k] > mx.v[k]) mx.v[k] = v.v[k];
			if (v.v[k] < mn.v[k]) mn.v[k] = v.v[k];
		}
	}
	*min = mn;
	*max = mx;
}

/* the covered chunk range (voxelShapes.c:152-177): floor / ceil of the box, one voxel more each way when
 * removing, split with DN_separate_position (truncating division) and clamped to the map.  False when
 * it is empty. */
static bool chunk_range(const DNvolume* vol, DNvec3 min, DNvec3 max, bool removing, int32_t cmin[3], int32_t cmax[3])
{
	DNivec3 lo = {(int)floorf(min.x), (int)floorf(min.y), (int)floorf(min.z)};
	DNivec3 hi = {(int)ceilf(max.x), (int)ceilf(max.y), (int)ceilf(max.z)};
	if (removing) {
		lo = (DNivec3){lo.x - 1, lo.y - 1, lo.z - 1};
		hi = (DNivec3){hi.x + 1, hi.y + 1, hi.z + 1};
	}
	DNivec3 mlo, mhi, unused;
	DN_separate_position(lo, &mlo, &unused);
	DN_separate_position(hi, &mhi, &unused);
	const int size[3] = {(int)vol->mapSize.x, (int)vol->mapSize.y, (int)vol->mapSize.z};
	const int l[3] = {mlo.x, mlo.y, mlo.z}, h[3] = {mhi.x, mhi.y, mhi.z};
	for (int k = 0; k < 3; k++) {
		cmin[k] = l[k] > 0 ? l[k] : 0;
		cmax[k] = h[k] < size[k] - 1 ? h[k] : size[k] - 1;
		if (cmin[k] > cmax[k]) return false;
	}
	return true;
}

/* the voxel word at (tile t, cp) as DN_get_compressed_voxel reads it: empty where the tile has no chunk */
static inline DNcompressedVoxel word_at(const DNvolume* vol, size_t t, DNivec3 cp)
{
	const DNchunkHandle h = vol->map[t];
	if (!h.flag) return (DNcompressedVoxel){0xFFFFFFFFu, 0u};
	return vol->chunks[h.chunkIndex].voxels[cp.x][cp.y][cp.z];
}

/* Applies evaluated hits to the CPU map (exported for tests).  counts: per chunk of the range
 * [cmin, cmax] in x-fastest order; hits: concatenated in that chunk order.  Without a transform function
 * the rules are applied on the voxel words directly (DN_compress_voxel + DN_set_compressed_voxel, the
 * steps DN_get_voxel / DN_set_voxel take); with one, through DN_get_voxel / DN_set_voxel. */
void dn_shape_apply(DNvolume* vol, DNvoxel voxel, bool flipNormals, bool sphere, VoxelTransformFunc func,
                    void* userData, DNvec3 shapeMin, DNvec3 shapeMax, DNmat4 invTransform, const int32_t cmin[3],
                    const int32_t cmax[3], const uint32_t* counts, const dn_shape_hit* hits)
{
	(void)flipNormals;   /* shell hits are only produced when flipping */
	const bool removing = voxel.material == DN_MATERIAL_EMPTY;
	size_t chunk = 0;
	uint64_t at = 0;
	for (int32_t mz = cmin[2]; mz <= cmax[2]; mz++)
	for (int32_t my = cmin[1]; my <= cmax[1]; my++)
	for (int32_t mx = cmin[0]; mx <= cmax[0]; mx++) {
		const DNivec3 mapPos = {mx, my, mz};
		/* the tile as it was before this chunk's edits (voxelShapes.c:186) */
		const DNchunkHandle tile = vol->map[DN_FLATTEN_INDEX(mapPos, vol->mapSize)];
		const uint32_t n = counts[chunk++];
		const size_t t = DN_FLATTEN_INDEX(mapPos, vol->mapSize);
		if (!func) {
			/* the placed voxel's word with its own normal (removals store it as is) */
			const DNcompressedVoxel placed = DN_compress_voxel(voxel);
			for (uint32_t i = 0; i < n; i++) {
				const dn_shape_hit* e = &hits[at++];
				const DNivec3 cp = {e->local & 7, (e->local >> 3) & 7, e->local >> 6};
				const DNcompressedVoxel cur = word_at(vol, t, cp);
				const bool exists = (cur.normal >> 24) != DN_MATERIAL_EMPTY;
				DNvoxel v;
				if (e->inside) {
					if (tile.flag != 0 && exists && !removing) continue;
					if (removing) { DN_set_compressed_voxel(vol, mapPos, cp, placed); continue; }
					v = voxel;
					v.normal = (DNvec3){{e->normal[0], e->normal[1], e->normal[2]}};
				} else {
					if (tile.flag == 0 || !exists) continue;
					v = DN_decompress_voxel(cur);
					v.normal = DN_vec3_scale((DNvec3){{e->normal[0], e->normal[1], e->normal[2]}}, -1.0f);
				}
				DN_set_compressed_voxel(vol, mapPos, cp, DN_compress_voxel(v));
			}
			continue;
		}
		for (uint32_t i = 0; i < n; i++) {
			const dn_shape_hit* e = &hits[at++];
			const DNivec3 cp = {e->local & 7, (e->local >> 3) & 7, e->local >> 6};
			const DNvec3 pos = {{(float)(mx * DN_CHUNK_SIZE + cp.x), (float)(my * DN_CHUNK_SIZE + cp.y),
			                     (float)(mz * DN_CHUNK_SIZE + cp.z)}};
			const DNvec3 normal = {{e->normal[0], e->normal[1], e->normal[2]}};
			if (e->inside) {
				if (tile.flag != 0 && DN_does_voxel_exist(vol, mapPos, cp) && !removing) continue;
				DNvoxel fin = voxel;
				if (!removing) {
					if (func) fin = func(pos, normal, voxel, shapeMin, shapeMax, invTransform, userData);
					else fin.normal = normal;
				}
				DN_set_voxel(vol, mapPos, cp, fin);
			} else {
				if (tile.flag == 0 || !DN_does_voxel_exist(vol, mapPos, cp)) continue;
				DNvoxel old = DN_get_voxel(vol, mapPos, cp);
				const DNvec3 flipped = DN_vec3_scale(normal, -1.0f);
				if (func) old = func(pos, flipped, old, shapeMin, shapeMax, sphere ? invTransform : DN_mat4_identity(), userData);
				else old.normal = flipped;
				DN_set_voxel(vol, mapPos, cp, old);
			}
		}
	}
}

/* the common tail of every shape: bounds, range, device evaluation, edits */
static void run_shape(DNvolume* vol, DNvoxel voxel, bool flipNormals, VoxelTransformFunc func, void* userData,
                      DNvec3 min, DNvec3 max, DNmat4 transform, dn_shape_params* p, const char* who)
{
	if (!vol) return;
	const bool sphere = p->kind == DN_SHAPE_SPHERE;
	const DNmat4 inv = DN_mat4_inv(transform);
	if (!sphere) transform_bounds(&min, &max, transform);
	p->removing = voxel.material == DN_MATERIAL_EMPTY;
	p->flipNormals = flipNormals ? 1u : 0u;
	memcpy(p->invTransform, inv.m, sizeof(p->invTransform));
	if (!chunk_range(vol, min, max, p->removing != 0, p->chunkMin, p->chunkMax)) return;
	const size_t nchunks = (size_t)(p->chunkMax[0] - p->chunkMin[0] + 1) * (size_t)(p->chunkMax[1] - p->chunkMin[1] + 1) *
	                       (size_t)(p->chunkMax[2] - p->chunkMin[2] + 1);
	uint32_t* counts = (uint32_t*)malloc(nchunks * sizeof(uint32_t));
	if (!counts) { shape_msg(DN_MESSAGE_ERROR, "%s: out of host memory", who); return; }
	dn_shape_hit* hits = NULL;
	uint64_t total = 0;
	if (dn_cuda_shape_eval(p, counts, &hits, &total) != DN_CUDA_OK) {
		shape_msg(DN_MESSAGE_ERROR, "%s: shape evaluation failed: %s", who, dn_cuda_last_error());
		free(counts);
		return;
	}
	dn_shape_apply(vol, voxel, flipNormals, sphere, func, userData, min, max, inv, p->chunkMin, p->chunkMax, counts, hits);
	dn_cuda_shape_free(hits);
	free(counts);
}

static DNmat4 placed(DNvec3 at, DNquaternion orient)
{
	return DN_mat4_mult(DN_mat4_translate(at), DN_quaternion_to_mat4(orient));
}

void DN_shape_sphere(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, float r, DNquaternion orient,
                     VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:239-333: squared distance to the centre; the box is not transformed */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_SPHERE;
	p.center[0] = c.x; p.center[1] = c.y; p.center[2] = c.z;
	p.r2 = r * r;
	p.r12 = (r + 1.0f) * (r + 1.0f);
	const DNvec3 min = {{c.x - r, c.y - r, c.z - r}}, max = {{c.x + r, c.y + r, c.z + r}};
	run_shape(vol, voxel, flipNormals, func, userData, min, max, placed(c, orient), &p, "DN_shape_sphere");
}

void DN_shape_box(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, DNvec3 len, DNquaternion orient,
                  VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:335-344 */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_BOX;
	p.length[0] = len.x; p.length[1] = len.y; p.length[2] = len.z;
	run_shape(vol, voxel, flipNormals, func, userData, DN_vec3_scale(len, -1.0f), len, placed(c, orient), &p, "DN_shape_box");
}

void DN_shape_rounded_box(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, DNvec3 len, float r,
                          DNquaternion orient, VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:346-359; the box's upper corner uses len.x on every axis, as the reference does */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_ROUNDED_BOX;
	p.length[0] = len.x; p.length[1] = len.y; p.length[2] = len.z;
	p.radius = r;
	const DNvec3 min = {{-len.x - r, -len.y - r, -len.z - r}}, max = {{len.x + r, len.x + r, len.x + r}};
	run_shape(vol, voxel, flipNormals, func, userData, min, max, placed(c, orient), &p, "DN_shape_rounded_box");
}

void DN_shape_torus(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, float ra, float rb, DNquaternion orient,
                    VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:361-374 */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_TORUS;
	p.radius = ra;
	p.radiusB = rb;
	const DNvec3 min = {{-(ra + rb), -rb, -(ra + rb)}}, max = {{ra + rb, rb, ra + rb}};
	run_shape(vol, voxel, flipNormals, func, userData, min, max, placed(c, orient), &p, "DN_shape_torus");
}

void DN_shape_ellipsoid(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, DNvec3 r, DNquaternion orient,
                        VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:376-388 */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_ELLIPSOID;
	p.radii[0] = r.x; p.radii[1] = r.y; p.radii[2] = r.z;
	const DNvec3 min = {{-r.x, -r.y, -r.z}};
	run_shape(vol, voxel, flipNormals, func, userData, min, r, placed(c, orient), &p, "DN_shape_ellipsoid");
}

void DN_shape_cylinder(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, float r, float h, DNquaternion orient,
                       VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:390-403 */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_CYLINDER;
	p.radius = r;
	p.height = h / 2;
	const DNvec3 min = {{-r, -h / 2, -r}}, max = {{r, h / 2, r}};
	run_shape(vol, voxel, flipNormals, func, userData, min, max, placed(c, orient), &p, "DN_shape_cylinder");
}

void DN_shape_cone(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 b, float r, float h, DNquaternion orient,
                   VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:405-425: the apex sits h along the rotated up axis from the base centre b */
	const DNmat4 rot = DN_quaternion_to_mat4(orient);
	const DNvec4 up4 = DN_mat4_mult_vec4(rot, (DNvec4){{0.0f, 1.0f, 0.0f, 1.0f}});
	const DNvec3 up = {{up4.x, up4.y, up4.z}};
	const DNvec3 apex = DN_vec3_add(b, DN_vec3_scale(up, h));
	const DNmat4 transform = DN_mat4_mult(DN_mat4_translate(apex), rot);
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_CONE;
	const float hyp = sqrtf(r * r + h * h);
	p.angles[0] = h / hyp;
	p.angles[1] = r / hyp;
	p.height = h;
	const DNvec3 min = {{-r, -h, -r}}, max = {{r, 0.0f, r}};
	run_shape(vol, voxel, flipNormals, func, userData, min, max, transform, &p, "DN_shape_cone");
}

void DN_shape_pyramid(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 b, DNvec3 len, DNquaternion orient,
                      VoxelTransformFunc func, void* userData)
{
	/* voxelShapes.c:427-442 */
	dn_shape_params p;
	memset(&p, 0, sizeof(p));
	p.kind = DN_SHAPE_PYRAMID;
	p.length[0] = len.x; p.length[2] = len.z;
	p.height = len.y;
	const DNvec3 min = {{-len.x * 0.5f, 0.0f, -len.z * 0.5f}}, max = {{len.x * 0.5f, len.y, len.z * 0.5f}};
	run_shape(vol, voxel, flipNormals, func, userData, min, max, placed(b, orient), &p, "DN_shape_pyramid");
}
