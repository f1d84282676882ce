"""ctypes view of libdoonengine.so: the DN_* API (include/DoonEngine/voxel.h) and the dn_cuda_* C ABI
(include/dn_cuda.h).  Struct layouts mirror the C headers; ``check_layout()`` compares them with the
library's own ``DN_abi_layout``."""
import ctypes
import os
from ctypes import (POINTER, Structure, c_bool, c_char_p, c_double, c_float, c_int, c_size_t, c_uint8, c_uint32,
                    c_uint64, c_void_p, c_int32, c_int64)

from . import build as _build


class DNvec2(Structure):
    _fields_ = [("x", c_float), ("y", c_float)]


class DNvec3(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float)]

    def tolist(self):
        return [self.x, self.y, self.z]


class DNmat4(Structure):
    _fields_ = [("m", (c_float * 4) * 4)]   # column-major m[col][row]


class DNivec3(Structure):
    _fields_ = [("x", c_int32), ("y", c_int32), ("z", c_int32)]


class DNuvec3(Structure):
    _fields_ = [("x", c_uint32), ("y", c_uint32), ("z", c_uint32)]


class DNcolor(Structure):
    _fields_ = [("r", c_uint8), ("g", c_uint8), ("b", c_uint8)]


class DNvoxel(Structure):
    _fields_ = [("material", c_uint8), ("normal", DNvec3), ("albedo", DNcolor)]


class DNvec4(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("w", c_float)]


class DNquaternion(Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("w", c_float)]


class DNcompressedVoxel(Structure):
    _fields_ = [("normal", c_uint32), ("albedo", c_uint32)]


class DNchunk(Structure):
    _fields_ = [("pos", DNivec3), ("updated", c_bool), ("numVoxels", c_uint32), ("numVoxelsGpu", c_uint32),
                ("voxels", DNcompressedVoxel * 512)]   # [x][y][z] flattened: x*64 + y*8 + z


class DNchunkHandle(Structure):
    _fields_ = [("flag", c_uint8), ("chunkIndex", c_uint32)]


class DNmaterial(Structure):
    _fields_ = [("padding", DNvec2), ("emissive", c_uint32), ("opacity", c_float), ("refractIndex", c_float),
                ("specular", c_float), ("reflectType", c_uint32), ("shininess", c_uint32)]


class DNvolume(Structure):
    _fields_ = [
        ("gpu", c_void_p),
        ("mapSize", DNuvec3),
        ("chunkCap", c_size_t), ("nextChunk", c_size_t), ("voxelCap", c_size_t), ("numVoxelNodes", c_size_t),
        ("numLightingRequests", c_size_t), ("lightingRequestCap", c_size_t),
        ("map", POINTER(DNchunkHandle)), ("chunks", POINTER(DNchunk)), ("materials", POINTER(DNmaterial)),
        ("lightingRequests", POINTER(c_uint32)), ("gpuVoxelLayout", c_void_p),
        ("camPos", DNvec3), ("camOrient", DNvec3), ("camFOV", c_float), ("camViewMode", c_uint32),
        ("sunDir", DNvec3), ("sunStrength", DNvec3), ("ambientLightStrength", DNvec3),
        ("diffuseBounceLimit", c_uint32), ("specBounceLimit", c_uint32), ("shadowSoftness", c_float),
        ("useCubemap", c_bool), ("glCubemapTex", c_uint32), ("skyGradientBot", DNvec3), ("skyGradientTop", DNvec3),
        ("frameNum", c_uint32), ("lastTime", c_float),
        ("emissiveStrength", c_float), ("numDirectRays", c_uint32), ("rngMode", c_uint32), ("mapId", c_uint32),
        ("truncateDispatch", c_uint32), ("deviceBudgetBytes", c_uint64),
    ]


class DNimage(Structure):
    _fields_ = [("width", c_uint32), ("height", c_uint32), ("color", POINTER(c_float)),
                ("hitIndex", POINTER(c_uint32)), ("hitFace", POINTER(c_uint8)), ("onDevice", c_int)]


class DNstats(Structure):
    _fields_ = [("rays", c_uint64), ("primaryRays", c_uint64), ("outerSteps", c_uint64), ("chunksEntered", c_uint64),
                ("innerSteps", c_uint64), ("hits", c_uint64), ("litVoxels", c_uint64), ("degenerate", c_uint64)]


class DnLightParams(Structure):
    """dn_light_params of include/dn_cuda.h"""
    _fields_ = [("sunDir", c_float * 3), ("sunStrength", c_float * 3), ("ambient", c_float * 3), ("camPos", c_float * 3),
                ("skyBot", c_float * 3), ("skyTop", c_float * 3), ("shadowSoftness", c_float), ("time", c_float),
                ("emissiveStrength", c_float), ("numDiffuse", c_uint32), ("maxDiffuse", c_uint32),
                ("diffuseBounceLimit", c_uint32), ("specBounceLimit", c_uint32), ("K", c_uint32), ("rngMode", c_uint32),
                ("mapId", c_uint32), ("spherePts", (c_float * 3) * 64)]


class DnDrawParams(Structure):
    """dn_draw_params of include/dn_cuda.h"""
    _fields_ = [("origin", c_float * 3), ("dirMat", (c_float * 4) * 4), ("width", c_uint32), ("height", c_uint32),
                ("viewMode", c_uint32), ("truncate16", c_uint32), ("sunStrength", c_float * 3),
                ("skyBot", c_float * 3), ("skyTop", c_float * 3), ("emissiveStrength", c_float),
                ("invProj", (c_float * 4) * 4), ("rasterColor", c_void_p), ("rasterDepth", c_void_p),
                ("rasterColorW", c_uint32), ("rasterColorH", c_uint32), ("rasterDepthW", c_uint32),
                ("rasterDepthH", c_uint32), ("compose", c_uint32)]


MESSAGE_CALLBACK = ctypes.CFUNCTYPE(None, c_int, c_int, c_char_p)
VOLP = POINTER(DNvolume)

PHASE_DRAW, PHASE_SYNC, PHASE_LIGHT = 1, 2, 4


class DNbatchItem(Structure):
    """DNbatchItem of include/DoonEngine/voxel.h"""
    _fields_ = [("vol", VOLP), ("phases", c_uint32), ("output", POINTER(DNimage)), ("view", DNmat4),
                ("projection", DNmat4), ("op", c_int), ("lightingSplit", c_int), ("numDiffuseSamples", c_int),
                ("maxDiffuseSamples", c_int), ("time", c_float), ("rasterColorTexture", c_int),
                ("rasterDepthTexture", c_int)]


REQUEST_DRAW, REQUEST_RELIGHT, REQUEST_EDIT = 0, 1, 2


class DNvoxelEdit(Structure):
    """DNvoxelEdit of include/DoonEngine/serve.h"""
    _fields_ = [("mapPos", DNivec3), ("chunkPos", DNivec3), ("voxel", DNvoxel), ("remove", c_int)]


class DNrequest(Structure):
    """DNrequest of include/DoonEngine/serve.h"""
    _fields_ = [("kind", c_int), ("volume", c_uint32), ("output", POINTER(DNimage)), ("view", DNmat4),
                ("projection", DNmat4), ("numDiffuseSamples", c_int), ("maxDiffuseSamples", c_int), ("time", c_float),
                ("edits", POINTER(DNvoxelEdit)), ("numEdits", c_uint32), ("user", c_void_p),
                ("rasterColorTexture", c_int), ("rasterDepthTexture", c_int)]


class DNcompletion(Structure):
    """DNcompletion of include/DoonEngine/serve.h"""
    _fields_ = [("id", c_uint64), ("user", c_void_p), ("kind", c_int), ("volume", c_uint32), ("arrival", c_double),
                ("admitted", c_double), ("finished", c_double), ("ok", c_int)]


class DNserveConfig(Structure):
    _fields_ = [("deviceBudgetBytes", c_uint64), ("maxVolumesPerTick", c_uint32), ("maxTicksInFlight", c_uint32)]


class DNserveStats(Structure):
    _fields_ = [("submitted", c_uint64), ("completed", c_uint64), ("failed", c_uint64), ("ticks", c_uint64),
                ("items", c_uint64), ("evictions", c_uint64), ("restores", c_uint64), ("residentBytes", c_uint64),
                ("residentVolumes", c_uint32), ("admitSeconds", c_double), ("issueSeconds", c_double),
                ("deviceSeconds", c_double), ("evictedBytes", c_uint64), ("restoredBytes", c_uint64),
                ("evictSeconds", c_double), ("restoreSeconds", c_double)]


class DnBatchTuning(Structure):
    """dn_batch_tuning of include/dn_cuda.h"""
    _fields_ = [("streamBatch", c_uint32), ("blocksPerSM", c_uint32), ("useGraph", c_uint32), ("kernel", c_uint32),
                ("poolRays", c_uint32), ("diffuseBatch", c_uint32)]

# (name, restype, argtypes)
_SIGS = [
    ("DN_init", c_bool, []),
    ("DN_quit", None, []),
    ("DN_create_volume", VOLP, [DNuvec3, c_uint32]),
    ("DN_create_volume_cpu", VOLP, [DNuvec3, c_uint32]),
    ("DN_delete_volume", None, [VOLP]),
    ("DN_load_volume", VOLP, [c_char_p, c_uint32]),
    ("DN_save_volume", c_bool, [c_char_p, VOLP]),
    ("DN_set_view_projection_matrices", None, [VOLP, c_float, c_float, c_float, POINTER(DNmat4), POINTER(DNmat4)]),
    ("DN_draw", None, [VOLP, POINTER(DNimage), DNmat4, DNmat4, c_int, c_int]),
    ("DN_update_lighting", None, [VOLP, c_int, c_int, c_float]),
    ("DN_add_chunk", c_int, [VOLP, DNivec3]),
    ("DN_remove_chunk", None, [VOLP, DNivec3]),
    ("DN_sync_gpu", None, [VOLP, c_int, c_int]),
    ("DN_set_map_size", c_bool, [VOLP, DNuvec3]),
    ("DN_set_max_chunks", c_bool, [VOLP, c_size_t]),
    ("DN_set_max_voxels_gpu", c_bool, [VOLP, c_size_t]),
    ("DN_set_residency", c_bool, [VOLP, c_int]),
    ("DN_get_residency", c_int, [VOLP]),
    ("DN_residency_nodes", c_size_t, [VOLP, POINTER(c_size_t), POINTER(c_uint32), POINTER(c_uint64),
                                      POINTER(c_int64), c_size_t]),
    ("DN_set_max_lighting_requests", c_bool, [VOLP, c_size_t]),
    ("DN_in_map_bounds", c_bool, [VOLP, DNivec3]),
    ("DN_in_chunk_bounds", c_bool, [DNivec3]),
    ("DN_get_voxel", DNvoxel, [VOLP, DNivec3, DNivec3]),
    ("DN_get_compressed_voxel", DNcompressedVoxel, [VOLP, DNivec3, DNivec3]),
    ("DN_set_voxel", None, [VOLP, DNivec3, DNivec3, DNvoxel]),
    ("DN_set_compressed_voxel", None, [VOLP, DNivec3, DNivec3, DNcompressedVoxel]),
    ("DN_remove_voxel", None, [VOLP, DNivec3, DNivec3]),
    ("DN_does_chunk_exist", c_bool, [VOLP, DNivec3]),
    ("DN_does_voxel_exist", c_bool, [VOLP, DNivec3, DNivec3]),
    ("DN_step_map", c_bool, [VOLP, DNvec3, DNvec3, c_int, POINTER(DNivec3), POINTER(DNvoxel), POINTER(DNivec3)]),
    ("DN_separate_position", None, [DNivec3, POINTER(DNivec3), POINTER(DNivec3)]),
    ("DN_cam_dir", DNvec3, [DNvec3]),
    ("DN_compress_voxel", DNcompressedVoxel, [DNvoxel]),
    ("DN_decompress_voxel", DNvoxel, [DNcompressedVoxel]),
    ("DN_finish", c_bool, [VOLP]),
    ("DN_image_create", POINTER(DNimage), [c_uint32, c_uint32, c_int, c_int]),
    ("DN_texture_create", c_int, [c_uint32, c_uint32, c_int]),
    ("DN_texture_destroy", None, [c_int]),
    ("DN_texture_upload", c_bool, [c_int, c_void_p]),
    ("DN_texture_format", c_int, [c_int]),
    ("DN_texture_device_pointer", c_void_p, [c_int, POINTER(c_uint32), POINTER(c_uint32)]),
    ("DN_image_destroy", None, [POINTER(DNimage)]),
    ("DN_draw_matrices", None, [DNmat4, DNmat4, POINTER(DNmat4), POINTER(DNmat4), POINTER(DNmat4)]),
    ("DN_get_stats", c_bool, [VOLP, POINTER(DNstats)]),
    ("DN_reset_stats", None, [VOLP]),
    ("DN_export_lighting", c_size_t, [VOLP, POINTER(c_uint32), POINTER(c_float), POINTER(c_float), c_size_t]),
    ("DN_export_tiles", c_bool, [VOLP, POINTER(c_uint8), POINTER(c_uint8), POINTER(c_uint32), POINTER(c_uint32)]),
    ("DN_export_requests", c_size_t, [VOLP, POINTER(c_uint32), c_size_t]),
    ("DN_compress_chunk", c_size_t, [VOLP, POINTER(DNchunk), POINTER(c_uint8)]),
    ("DN_decompress_chunk", c_int, [VOLP, POINTER(c_uint8), c_size_t, POINTER(DNchunk)]),
    ("DN_abi_layout", c_size_t, [POINTER(c_uint64), c_size_t]),
    ("DN_set_allocator", None, [c_void_p, c_void_p, c_void_p]),
    ("DN_mat4_inv", DNmat4, [DNmat4]),
    ("DN_mat4_mult", DNmat4, [DNmat4, DNmat4]),
    ("DN_mat4_translate", DNmat4, [DNvec3]),
    ("DN_mat4_mult_vec4", DNvec4, [DNmat4, DNvec4]),
    ("DN_vec3_add", DNvec3, [DNvec3, DNvec3]),
    ("DN_vec3_scale", DNvec3, [DNvec3, c_float]),
    ("DN_quaternion_identity", DNquaternion, []),
    ("DN_quaternion_from_euler", DNquaternion, [DNvec3]),
    ("DN_quaternion_to_mat4", DNmat4, [DNquaternion]),
    ("DN_shape_sphere", None, [VOLP, DNvoxel, c_bool, DNvec3, c_float, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_box", None, [VOLP, DNvoxel, c_bool, DNvec3, DNvec3, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_rounded_box", None, [VOLP, DNvoxel, c_bool, DNvec3, DNvec3, c_float, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_torus", None, [VOLP, DNvoxel, c_bool, DNvec3, c_float, c_float, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_ellipsoid", None, [VOLP, DNvoxel, c_bool, DNvec3, DNvec3, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_cylinder", None, [VOLP, DNvoxel, c_bool, DNvec3, c_float, c_float, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_cone", None, [VOLP, DNvoxel, c_bool, DNvec3, c_float, c_float, DNquaternion, c_void_p, c_void_p]),
    ("DN_shape_pyramid", None, [VOLP, DNvoxel, c_bool, DNvec3, DNvec3, DNquaternion, c_void_p, c_void_p]),
    ("DN_export_voxels", None, [VOLP, c_void_p, c_void_p, c_void_p]),
    ("dn_shape_apply", None, [VOLP, DNvoxel, c_bool, c_bool, c_void_p, c_void_p, DNvec3, DNvec3, DNmat4, c_void_p,
                              c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_shape_eval", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_shape_free", None, [c_void_p]),
    ("dn_cuda_shape_stats", None, [POINTER(c_uint64), POINTER(c_double), c_int]),
    ("DN_vec3_normalize", DNvec3, [DNvec3]),
    ("DN_batch_create", c_void_p, []),
    ("DN_batch_destroy", None, [c_void_p]),
    ("DN_batch_add", c_bool, [c_void_p, VOLP]),
    ("DN_batch_remove", c_bool, [c_void_p, VOLP]),
    ("DN_batch_run", c_bool, [c_void_p, POINTER(DNbatchItem), c_uint32]),
    ("DN_batch_finish", c_bool, [c_void_p]),
    ("DN_batch_get_stats", c_bool, [c_void_p, POINTER(DNstats)]),
    ("DN_batch_reset_stats", None, [c_void_p]),
    ("DN_batch_autotune", c_bool, [c_void_p]),
    ("DN_batch_stream", c_void_p, [c_void_p]),
    ("DN_server_create", c_void_p, [POINTER(DNserveConfig)]),
    ("DN_server_destroy", None, [c_void_p]),
    ("DN_server_add_volume", c_int, [c_void_p, VOLP]),
    ("DN_server_start", c_bool, [c_void_p]),
    ("DN_server_submit", c_uint64, [c_void_p, POINTER(DNrequest)]),
    ("DN_server_replay", c_size_t, [c_void_p, POINTER(DNrequest), POINTER(c_double), c_size_t]),
    ("DN_server_drain", c_bool, [c_void_p, c_double]),
    ("DN_server_poll", c_size_t, [c_void_p, POINTER(DNcompletion), c_size_t]),
    ("DN_server_get_stats", None, [c_void_p, POINTER(DNserveStats)]),
    ("DN_server_batch", c_void_p, [c_void_p]),
    ("DN_server_clock", c_double, []),
    ("dn_pack_chunk", c_uint32, [VOLP, POINTER(DNchunk), c_void_p, c_void_p, c_void_p]),
    ("dn_count_surface", c_uint32, [VOLP, POINTER(DNchunk)]),
    ("dn_scene_palette", None, [VOLP, c_uint32, c_uint32, c_uint32, c_float, c_float, c_float]),
    ("dn_scene_terrain", None, [VOLP, c_uint32, c_float, c_float, c_uint32, c_uint32]),
    ("dn_scene_shapes", None, [VOLP, c_uint32, c_uint32, c_int32, c_int32, c_uint32, c_float, c_float]),
    ("dn_scene_camera", None, [VOLP, c_float, c_float, c_float, c_float, c_float, c_float]),
    ("dn_scene_reroll", None, [VOLP, c_void_p, c_uint32, c_uint32, c_uint32]),
    # C ABI
    ("dn_cuda_init", c_int, [c_int]),
    ("dn_cuda_shutdown", None, []),
    ("dn_cuda_error_string", c_char_p, [c_int]),
    ("dn_cuda_last_error", c_char_p, []),
    ("dn_cuda_map_create", c_int, [c_uint32, c_uint32, c_uint32, c_uint32, c_uint64, POINTER(c_void_p)]),
    ("dn_cuda_map_destroy", None, [c_void_p]),
    ("dn_cuda_map_resize", c_int, [c_void_p, c_uint32, c_uint32, c_uint32]),
    ("dn_cuda_reserve", c_int, [c_void_p, c_uint32, c_uint64, c_uint64]),
    ("dn_cuda_sync", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_uint64]),
    ("dn_cuda_light", c_int, [c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_light_noalloc", c_int, [c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_light_noalloc_set_limit", c_uint32, [c_uint32]),
    ("dn_cuda_draw", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_draw_host", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_finish", c_int, [c_void_p, POINTER(c_uint64)]),
    ("dn_cuda_stats", c_int, [c_void_p, c_void_p]),
    ("dn_cuda_stats_kind", c_int, [c_void_p, c_int, c_void_p]),
    ("dn_cuda_reset_stats", c_int, [c_void_p]),
    ("dn_cuda_stream", c_void_p, [c_void_p]),
    ("dn_cuda_export_tiles", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_read_tile_flags", c_int, [c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_export_requests", c_int, [c_void_p, c_void_p, c_uint64, POINTER(c_uint64)]),
    ("dn_cuda_export_lighting", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint64, POINTER(c_uint64)]),
    ("dn_cuda_malloc", c_int, [POINTER(c_void_p), c_size_t]),
    ("dn_cuda_free", c_int, [c_void_p]),
    ("dn_cuda_malloc_host", c_int, [POINTER(c_void_p), c_size_t]),
    ("dn_cuda_free_host", c_int, [c_void_p]),
    ("dn_cuda_memcpy_d2h", c_int, [c_void_p, c_void_p, c_size_t]),
    ("dn_cuda_memcpy_h2d", c_int, [c_void_p, c_void_p, c_size_t]),
    ("dn_cuda_event_create", c_int, [POINTER(c_void_p)]),
    ("dn_cuda_event_destroy", c_int, [c_void_p]),
    ("dn_cuda_event_record", c_int, [c_void_p, c_void_p]),
    ("dn_cuda_event_elapsed_ms", c_int, [c_void_p, c_void_p, POINTER(c_float)]),
    ("dn_cuda_stream_sync", c_int, [c_void_p]),
    ("dn_cuda_device_sync", c_int, []),
    ("dn_cuda_flush_l2", c_int, [c_void_p, c_size_t]),
    ("dn_cuda_sync_stage", c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_uint64]),
    ("dn_cuda_sync_chunks", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p]),
    ("dn_cuda_sync_stage_chunks", c_int, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p]),
    ("dn_cuda_export_chunk", c_int, [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]),
    ("dn_cuda_stage_part_limit", c_size_t, [c_size_t]),
    ("dn_cuda_batch_create", c_int, [POINTER(c_void_p)]),
    ("dn_cuda_batch_destroy", None, [c_void_p]),
    ("dn_cuda_batch_add", c_int, [c_void_p, c_void_p]),
    ("dn_cuda_batch_remove", c_int, [c_void_p, c_void_p]),
    ("dn_cuda_batch_frame", c_int, [c_void_p, c_void_p, c_uint32]),
    ("dn_cuda_batch_finish", c_int, [c_void_p]),
    ("dn_cuda_batch_stats", c_int, [c_void_p, c_int, c_void_p]),
    ("dn_cuda_batch_reset_stats", c_int, [c_void_p]),
    ("dn_cuda_batch_stream", c_void_p, [c_void_p]),
    ("dn_cuda_batch_get_tuning", c_int, [c_void_p, POINTER(DnBatchTuning)]),
    ("dn_cuda_batch_set_tuning", c_int, [c_void_p, POINTER(DnBatchTuning)]),
    ("dn_cuda_batch_autotune", c_int, [c_void_p, POINTER(DnBatchTuning)]),
    ("dn_cuda_requests_of", c_uint64, [c_void_p]),
    ("dn_cuda_map_footprint", c_uint64, [c_void_p]),
    ("dn_cuda_map_is_resident", c_int, [c_void_p]),
    ("dn_cuda_map_evict", c_int, [c_void_p]),
    ("dn_cuda_map_restore", c_int, [c_void_p]),
    ("dn_cuda_map_restore_async", c_int, [c_void_p]),
    ("dn_cuda_map_restore_query", c_int, [c_void_p]),
    ("dn_cuda_host_reserve", c_int, [c_uint64]),
    ("dn_cuda_host_pinned", c_uint64, []),
    ("dn_cuda_host_pinned_free", c_uint64, []),
    ("dn_cuda_host_headroom", c_int, [c_uint64]),
    ("dn_cuda_host_slab_bytes", c_uint64, []),
    ("dn_cuda_event_query", c_int, [c_void_p]),
    ("dn_cuda_kernel_names", c_char_p, []),
    ("dn_cuda_launch_count", c_uint64, []),
    ("dn_cuda_alloc_count", c_uint64, []),
]

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libdoonengine.so (building it in-tree when it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libdoonengine.so is not built (%s); run doonengine_gb300.build.build()" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGS:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_names():
    return [n for n, _, _ in _SIGS]


def check_layout(lib=None):
    """Compare the ctypes struct layouts with the library's own sizes / offsets; returns a list of mismatches."""
    lib = lib or load()
    buf = (c_uint64 * 64)()
    n = lib.DN_abi_layout(buf, 64)
    want = [ctypes.sizeof(DNvolume), DNvolume.mapSize.offset, DNvolume.map.offset, DNvolume.chunks.offset,
            DNvolume.materials.offset, DNvolume.camPos.offset, DNvolume.sunDir.offset, DNvolume.useCubemap.offset,
            DNvolume.frameNum.offset, DNvolume.emissiveStrength.offset, DNvolume.deviceBudgetBytes.offset,
            ctypes.sizeof(DNchunk), ctypes.sizeof(DNmaterial), ctypes.sizeof(DNimage), ctypes.sizeof(DNchunkHandle),
            ctypes.sizeof(DNstats), DNchunk.voxels.offset, ctypes.sizeof(DNvoxel),
            ctypes.sizeof(DNbatchItem), DNbatchItem.view.offset, DNbatchItem.op.offset, DNbatchItem.time.offset,
            ctypes.sizeof(DNrequest), DNrequest.edits.offset, DNrequest.user.offset, ctypes.sizeof(DNcompletion),
            ctypes.sizeof(DNvoxelEdit), ctypes.sizeof(DNserveStats), DNbatchItem.rasterColorTexture.offset,
            DNrequest.rasterColorTexture.offset, ctypes.sizeof(DnDrawParams), DnDrawParams.compose.offset,
            ctypes.sizeof(DnLightParams)]
    return [(i, int(buf[i]), w) for i, w in enumerate(want[:n]) if int(buf[i]) != w]
