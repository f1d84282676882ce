/*
 * dn_residency.h -- host model of the reference's GPU voxel buffer (DN_RESIDENCY_LRU).
 *
 * The reference keeps every loaded chunk's voxels in one GL buffer cut into power-of-two nodes of
 * 16..512 voxels (voxel.c:1538-1640, DNvoxelNode in voxel.h:74-79).  A requested chunk takes the
 * smallest free node that fits, else the node of the loaded chunk unused for the most syncs; a chunk
 * touched in the last sync keeps its node, and with no node to take the chunk stays unloaded and the
 * buffer doubles at the end of the sync (voxel.c:773-781).  After the per-tile loop a bounded bubble
 * pass moves used nodes forward and merges equal free neighbours (voxel.c:1642-1695).
 *
 * This model reproduces those decisions -- which chunk loads, which one is unloaded, when the buffer
 * grows -- so that the visible residency of every tile is the reference's.  The voxel data itself stays
 * in the device pool's record slots; the nodes only decide.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dn_node {
	uint32_t size;     /* voxels, a power of two in 16..512 */
	uint64_t start;    /* first voxel */
	int64_t tile;      /* owning tile, -1 when free (the reference's chunkPos.x = -1) */
} dn_node;

typedef struct dn_nodes {
	dn_node* v;
	size_t n, cap;     /* nodes in buffer order; allocated entries */
	uint64_t voxelCap; /* buffer size in voxels */
} dn_nodes;

/* the buffer DN_create_volume makes for minChunks chunk slots (voxel.c:181, 190, 235-249) */
int dn_nodes_init(dn_nodes* b, uint64_t numChunks);
void dn_nodes_free(dn_nodes* b);
/* DN_set_max_voxels_gpu's node part (voxel.c:1031-1082): whole 512-voxel nodes appended */
int dn_nodes_grow(dn_nodes* b, uint64_t num);
/* _DN_unload_voxels (voxel.c:1538-1546): the first node owned by 'tile' becomes free */
void dn_nodes_unload(dn_nodes* b, int64_t tile);
/* _DN_stream_voxels' node choice (voxel.c:1554-1630) for a chunk of nvox voxels; lastUsed is read for
 * the tiles owning candidate nodes.  Returns 1 when the chunk got a node (*victim: the tile whose node
 * was taken, or -1), 0 when it did not (the buffer must grow).  -1 on allocation failure. */
int dn_nodes_stream(dn_nodes* b, int64_t tile, uint32_t nvox, const uint32_t* lastUsed, int64_t* victim);
/* _DN_sort_gpu_voxel_buffer (voxel.c:1642-1695) with at most maxCopies swaps and merges (the 11th ends it) */
void dn_nodes_sort(dn_nodes* b, int maxCopies);

#ifdef __cplusplus
}
#endif
