/*
 * voxelShapes.h -- shapes placed into a volume by signed distance (the reference's
 * src/DoonEngine/voxelShapes.h:1-161, shape functions).
 *
 * Same functions, arguments and results as the reference: every voxel of the chunks a shape's bounding
 * box covers is tested against the shape's distance function; voxels inside (distance < 0) are set to
 * the given voxel with a normal from the distance field (or the transform function's result).  Placing
 * DN_MATERIAL_EMPTY removes voxels; with flipNormals the existing voxels within distance 1 of the removed
 * region take the flipped normal.  The per-voxel distance and normal evaluation runs on the GPU (one
 * thread per voxel of the covered chunks); the edits are applied to the CPU map in the reference's order,
 * so the map (and the next DN_sync_gpu) sees exactly the reference's voxels.  A usable GPU is needed
 * (DN_init); the volume itself may be a CPU-only one (DN_create_volume_cpu).
 *
 * Not included: the MagicaVoxel model loader and model helpers of the reference's header
 * (DN_load_vox_file, DN_calculate_model_normals, DN_place_model_into_volume).
 */
#ifndef DN_VOXEL_SHAPES_H
#define DN_VOXEL_SHAPES_H

#include "voxel.h"

#ifdef __cplusplus
extern "C"
{
#endif

/* voxelShapes.h:25-34: computes the voxel actually placed.  pos in voxels; normal as computed (flipped for
 * the voxels next to a removal); shapeMin / shapeMax the transformed bounding box; invTransform into the
 * shape's local space (the identity for the flipped voxels of every shape but the sphere, as in the
 * reference) */
typedef DNvoxel (*VoxelTransformFunc)(DNvec3 pos, DNvec3 normal, DNvoxel vox, DNvec3 shapeMin, DNvec3 shapeMax,
                                      DNmat4 invTransform, void* userData);

/* voxelShapes.h:36-137; orientations are quaternions (DN_quaternion_identity / DN_quaternion_from_euler) */
void DN_shape_sphere(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, float r, DNquaternion orient,
                     VoxelTransformFunc func, void* userData);
void DN_shape_box(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, DNvec3 len, DNquaternion orient,
                  VoxelTransformFunc func, void* userData);
void DN_shape_rounded_box(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, DNvec3 len, float r,
                          DNquaternion orient, VoxelTransformFunc func, void* userData);
void DN_shape_torus(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, float ra, float rb, DNquaternion orient,
                    VoxelTransformFunc func, void* userData);
void DN_shape_ellipsoid(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, DNvec3 r, DNquaternion orient,
                        VoxelTransformFunc func, void* userData);
void DN_shape_cylinder(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 c, float r, float h, DNquaternion orient,
                       VoxelTransformFunc func, void* userData);
void DN_shape_cone(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 b, float r, float h, DNquaternion orient,
                   VoxelTransformFunc func, void* userData);
void DN_shape_pyramid(DNvolume* vol, DNvoxel voxel, bool flipNormals, DNvec3 b, DNvec3 len, DNquaternion orient,
                      VoxelTransformFunc func, void* userData);

/* addition, for tests and tools: the host half of a shape call -- applies evaluated hits (the output of
 * dn_cuda_shape_eval for the chunk range [cmin, cmax]) to the CPU map with the reference's rules */
struct dn_shape_hit;
void dn_shape_apply(DNvolume* vol, DNvoxel voxel, bool flipNormals, bool sphere, VoxelTransformFunc func,
                    void* userData, DNvec3 shapeMin, DNvec3 shapeMax, DNmat4 invTransform, const int32_t cmin[3],
                    const int32_t cmax[3], const uint32_t* counts, const struct dn_shape_hit* hits);

#ifdef __cplusplus
}
#endif

#endif
