/*
 * dnref_shim.c -- TEST INFRASTRUCTURE.  Compiles the reference's own host C,
 * src/DoonEngine/voxel.c, unchanged from where it lies in the reference tree
 * (the include path is set by oracle/ref/Makefile), and exports its pure-CPU
 * functions so that golden vectors can be generated from the reference
 * itself.
 *
 * Everything defined by voxel.c is compiled with hidden visibility and the
 * library is linked with --gc-sections and --no-undefined: functions that
 * touch OpenGL (DN_init, DN_create_volume, DN_draw, DN_sync_gpu, ...) are
 * never referenced, so they are dropped at link time and no GL symbol,
 * loader or library is involved.  The link fails if any GL reference
 * survives.  x86-64 only: the reference's vendored math header forces SSE.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "voxel.c"
#include "voxelShapes.c"

#define EXPORT __attribute__((visibility("default")))

static void ref_silent(DNmessageType t, DNmessageSeverity s, const char* m) { (void)t; (void)s; (void)m; }

EXPORT uint32_t ref_sizeof_chunk(void) { return (uint32_t)sizeof(DNchunk); }
EXPORT uint32_t ref_sizeof_volume(void) { return (uint32_t)sizeof(DNvolume); }

/* voxel.c:1289-1316 */
EXPORT void ref_compress_voxel(uint8_t material, const float normal[3], const uint8_t albedo[3], uint32_t out[2])
{
    DNvoxel v;
    v.material = material;
    v.normal = (DNvec3){{normal[0], normal[1], normal[2]}};
    v.albedo = (DNcolor){albedo[0], albedo[1], albedo[2]};
    DNcompressedVoxel c = DN_compress_voxel(v);
    out[0] = c.normal; out[1] = c.albedo;
}

EXPORT void ref_decompress_voxel(const uint32_t in[2], uint8_t* material, float normal[3], uint8_t albedo[3])
{
    DNcompressedVoxel c = {in[0], in[1]};
    DNvoxel v = DN_decompress_voxel(c);
    *material = v.material;
    normal[0] = v.normal.x; normal[1] = v.normal.y; normal[2] = v.normal.z;
    albedo[0] = v.albedo.r; albedo[1] = v.albedo.g; albedo[2] = v.albedo.b;
}

/* voxel.c:1397-1461: mask[16], partial[3], nvox, voxels[n][2] (normal, linear albedo) */
EXPORT void ref_chunk_to_gpu(const DNchunk* chunk, const DNmaterial* materials, uint32_t mask[16],
                             uint32_t partial[3], uint32_t* nvox, uint32_t voxels[512][2])
{
    DNvolume vol;
    memset(&vol, 0, sizeof(vol));
    vol.materials = (DNmaterial*)materials;
    int n = 0;
    static DNvoxelGPU tmp[DN_CHUNK_LENGTH];
    DNchunkGPU g = _DN_chunk_to_gpu(&vol, *chunk, &n, tmp);
    memcpy(mask, g.bitMask, sizeof(g.bitMask));
    memcpy(partial, g.partialCounts, sizeof(g.partialCounts));
    *nvox = (uint32_t)n;
    for (int i = 0; i < n; i++) { voxels[i][0] = tmp[i].normal; voxels[i][1] = tmp[i].directLight; }
}

/* camera: voxel.c:788-810 and the inverses of voxel.c:845-853 */
EXPORT void ref_view_projection(const float camPos[3], const float camOrient[3], float fov, float aspect,
                                float nearPlane, float farPlane, float view[16], float proj[16],
                                float invView[16], float invCenteredView[16], float invProj[16])
{
    DNvolume vol;
    memset(&vol, 0, sizeof(vol));
    vol.camPos = (DNvec3){{camPos[0], camPos[1], camPos[2]}};
    vol.camOrient = (DNvec3){{camOrient[0], camOrient[1], camOrient[2]}};
    vol.camFOV = fov;
    DNmat4 v, p;
    DN_set_view_projection_matrices(&vol, aspect, nearPlane, farPlane, &v, &p);
    DNmat4 cv = v;
    cv.m[3][0] = 0.0f; cv.m[3][1] = 0.0f; cv.m[3][2] = 0.0f;
    DNmat4 iv = DN_mat4_inv(v), icv = DN_mat4_inv(cv), ip = DN_mat4_inv(p);
    memcpy(view, v.m, 64); memcpy(proj, p.m, 64);
    memcpy(invView, iv.m, 64); memcpy(invCenteredView, icv.m, 64); memcpy(invProj, ip.m, 64);
}

EXPORT void ref_cam_dir(const float orient[3], float out[3])
{
    DNvec3 d = DN_cam_dir((DNvec3){{orient[0], orient[1], orient[2]}});
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

EXPORT void ref_vec3_normalize(const float in[3], float out[3])
{
    DNvec3 d = DN_vec3_normalize((DNvec3){{in[0], in[1], in[2]}});
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

/* A volume holding only the CPU-side arrays that DN_create_volume sets up
 * (voxel.c:199-278); no GPU buffer is created. */
EXPORT DNvolume* ref_volume_new(uint32_t sx, uint32_t sy, uint32_t sz, uint32_t minChunks)
{
    g_DN_message_callback = ref_silent;
    DNvolume* vol = (DNvolume*)calloc(1, sizeof(DNvolume));
    size_t tiles = (size_t)sx * sy * sz;
    size_t n = tiles < minChunks ? tiles : minChunks;
    vol->map = (DNchunkHandle*)calloc(tiles, sizeof(DNchunkHandle));
    vol->chunks = (DNchunk*)malloc(sizeof(DNchunk) * n);
    vol->materials = (DNmaterial*)calloc(DN_MAX_MATERIALS, sizeof(DNmaterial));
    vol->mapSize = (DNuvec3){sx, sy, sz};
    vol->chunkCap = n;
    vol->nextChunk = 0;
    for (size_t i = 0; i < n; i++) _DN_clear_chunk(vol, (int)i);
    return vol;
}

EXPORT void ref_volume_free(DNvolume* vol)
{
    free(vol->map); free(vol->chunks); free(vol->materials); free(vol);
}

EXPORT void ref_volume_info(const DNvolume* vol, uint64_t out[3])
{
    out[0] = vol->chunkCap; out[1] = vol->nextChunk; out[2] = 0;
}

EXPORT DNchunkHandle* ref_volume_map(DNvolume* vol) { return vol->map; }
EXPORT DNchunk* ref_volume_chunks(DNvolume* vol) { return vol->chunks; }

EXPORT void ref_set_voxel(DNvolume* vol, const int32_t mapPos[3], const int32_t chunkPos[3],
                          uint8_t material, const float normal[3], const uint8_t albedo[3])
{
    DNvoxel v;
    v.material = material;
    v.normal = (DNvec3){{normal[0], normal[1], normal[2]}};
    v.albedo = (DNcolor){albedo[0], albedo[1], albedo[2]};
    DN_set_voxel(vol, (DNivec3){mapPos[0], mapPos[1], mapPos[2]}, (DNivec3){chunkPos[0], chunkPos[1], chunkPos[2]}, v);
}

EXPORT void ref_set_compressed_voxel(DNvolume* vol, const int32_t mapPos[3], const int32_t chunkPos[3], const uint32_t v[2])
{
    DNcompressedVoxel c = {v[0], v[1]};
    DN_set_compressed_voxel(vol, (DNivec3){mapPos[0], mapPos[1], mapPos[2]}, (DNivec3){chunkPos[0], chunkPos[1], chunkPos[2]}, c);
}

EXPORT void ref_remove_voxel(DNvolume* vol, const int32_t mapPos[3], const int32_t chunkPos[3])
{
    DN_remove_voxel(vol, (DNivec3){mapPos[0], mapPos[1], mapPos[2]}, (DNivec3){chunkPos[0], chunkPos[1], chunkPos[2]});
}

EXPORT int ref_step_map(DNvolume* vol, const float dir[3], const float pos[3], int maxSteps,
                        int32_t hitPos[3], uint32_t hitVoxel[2], int32_t hitNormal[3])
{
    DNivec3 hp = {0, 0, 0}, hn;
    DNvoxel hv;
    memset(&hv, 0, sizeof(hv));
    bool r = DN_step_map(vol, (DNvec3){{dir[0], dir[1], dir[2]}}, (DNvec3){{pos[0], pos[1], pos[2]}}, maxSteps, &hp, &hv, &hn);
    hitPos[0] = hp.x; hitPos[1] = hp.y; hitPos[2] = hp.z;
    hitNormal[0] = hn.x; hitNormal[1] = hn.y; hitNormal[2] = hn.z;
    DNcompressedVoxel c = DN_compress_voxel(hv);
    hitVoxel[0] = c.normal; hitVoxel[1] = c.albedo;
    return r ? 1 : 0;
}

/* .voxvol chunk codec, voxel.c:301-518 */
EXPORT uint32_t ref_compress_chunk(DNvolume* vol, const DNchunk* chunk, char* mem)
{
    return _DN_compress_chunk(*chunk, vol, mem);
}

EXPORT void ref_decompress_chunk(DNvolume* vol, const char* mem, DNchunk* out)
{
    _DN_decompress_chunk((char*)mem, vol, out);
}

/* ---- shapes, voxelShapes.c:239-442 ---- */

/* one shape call: kind 0 sphere (c, a = r), 1 box (c, v = len), 2 rounded box (c, v, a = r), 3 torus
 * (c, a = ra, b = rb), 4 ellipsoid (c, v = radii), 5 cylinder (c, a = r, b = h), 6 cone (base c, a = r,
 * b = h), 7 pyramid (base c, v = len); orientation from Euler angles in degrees */
typedef struct ref_shape_op {
    int32_t kind, flip, transform;   /* transform: 1 passes ref_shape_transform as the transform function */
    uint8_t material, albedo[3];
    float normal[3], c[3], v[3], a, b, euler[3];
} ref_shape_op;

/* the transform function of the shape tests: colour from the position in shape space, material from the
 * side the normal faces, the normal kept */
static DNvoxel ref_shape_transform(DNvec3 pos, DNvec3 normal, DNvoxel vox, DNvec3 mn, DNvec3 mx, DNmat4 inv, void* user)
{
    (void)user;
    DNvec4 lp = DN_mat4_mult_vec4(inv, (DNvec4){{pos.x, pos.y, pos.z, 1.0f}});
    vox.normal = normal;
    vox.albedo.r = (uint8_t)((int)floorf(lp.x * 8.0f) & 255);
    vox.albedo.g = (uint8_t)((int)floorf(lp.y * 8.0f) & 255);
    vox.albedo.b = (uint8_t)((int)floorf((pos.z - mn.z) * 4.0f + mx.x) & 255);
    vox.material = normal.y > 0.0f ? 3 : 4;
    return vox;
}

EXPORT void ref_shape_run(DNvolume* vol, const ref_shape_op* op)
{
    DNvoxel vox;
    vox.material = op->material;
    vox.normal = (DNvec3){{op->normal[0], op->normal[1], op->normal[2]}};
    vox.albedo = (DNcolor){op->albedo[0], op->albedo[1], op->albedo[2]};
    DNquaternion q = DN_quaternion_from_euler((DNvec3){{op->euler[0], op->euler[1], op->euler[2]}});
    DNvec3 c = {{op->c[0], op->c[1], op->c[2]}}, v = {{op->v[0], op->v[1], op->v[2]}};
    VoxelTransformFunc f = op->transform ? ref_shape_transform : NULL;
    switch (op->kind) {
    case 0: DN_shape_sphere(vol, vox, op->flip, c, op->a, q, f, NULL); break;
    case 1: DN_shape_box(vol, vox, op->flip, c, v, q, f, NULL); break;
    case 2: DN_shape_rounded_box(vol, vox, op->flip, c, v, op->a, q, f, NULL); break;
    case 3: DN_shape_torus(vol, vox, op->flip, c, op->a, op->b, q, f, NULL); break;
    case 4: DN_shape_ellipsoid(vol, vox, op->flip, c, v, q, f, NULL); break;
    case 5: DN_shape_cylinder(vol, vox, op->flip, c, op->a, op->b, q, f, NULL); break;
    case 6: DN_shape_cone(vol, vox, op->flip, c, op->a, op->b, q, f, NULL); break;
    case 7: DN_shape_pyramid(vol, vox, op->flip, c, v, q, f, NULL); break;
    }
}

/* the quaternion, translate * rotation and its inverse of a shape call (the cone's translation is its
 * apex), as DN_shape_* builds them */
EXPORT void ref_shape_matrices(const ref_shape_op* op, float q[4], float transform[16], float inv[16])
{
    DNquaternion qq = DN_quaternion_from_euler((DNvec3){{op->euler[0], op->euler[1], op->euler[2]}});
    DNmat4 rot = DN_quaternion_to_mat4(qq);
    DNvec3 at = {{op->c[0], op->c[1], op->c[2]}};
    if (op->kind == 6) {
        DNvec4 up = DN_mat4_mult_vec4(rot, (DNvec4){{0.0f, 1.0f, 0.0f, 1.0f}});
        at = DN_vec3_add(at, DN_vec3_scale((DNvec3){{up.x, up.y, up.z}}, op->b));
    }
    DNmat4 t = DN_mat4_mult(DN_mat4_translate(at), rot);
    DNmat4 it = DN_mat4_inv(t);
    memcpy(q, &qq, 16);
    memcpy(transform, t.m, 64);
    memcpy(inv, it.m, 64);
}

/* dense copy of the CPU map: normal word per voxel (0xFFFFFFFF where the tile has no chunk), albedo word
 * (0 for empty voxels), flag per tile */
EXPORT void ref_export_voxels(const DNvolume* vol, uint32_t* normalWords, uint32_t* albedoWords, uint8_t* tileFlags)
{
    const uint32_t X = vol->mapSize.x * 8, Y = vol->mapSize.y * 8;
    for (uint32_t tz = 0; tz < vol->mapSize.z; tz++)
    for (uint32_t ty = 0; ty < vol->mapSize.y; ty++)
    for (uint32_t tx = 0; tx < vol->mapSize.x; tx++) {
        const size_t t = tx + (size_t)vol->mapSize.x * (ty + (size_t)vol->mapSize.y * tz);
        tileFlags[t] = vol->map[t].flag;
        const DNchunk* c = vol->map[t].flag ? &vol->chunks[vol->map[t].chunkIndex] : NULL;
        for (uint32_t z = 0; z < 8; z++)
        for (uint32_t y = 0; y < 8; y++)
        for (uint32_t x = 0; x < 8; x++) {
            const size_t i = (tx * 8 + x) + (size_t)X * ((ty * 8 + y) + (size_t)Y * (tz * 8 + z));
            const DNcompressedVoxel w = c ? c->voxels[x][y][z] : (DNcompressedVoxel){UINT32_MAX, 0};
            normalWords[i] = w.normal;
            albedoWords[i] = (w.normal >> 24) == DN_MATERIAL_EMPTY ? 0u : w.albedo;
        }
    }
}
