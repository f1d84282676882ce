/*
 * dn_residency.c -- host model of the reference's GPU voxel-buffer nodes (DN_RESIDENCY_LRU); the
 * decisions of voxel.c:1538-1695 on a node list, with no voxel data behind it.
 */
#include "dn_residency.h"
#include "DoonEngine/globals.h"
#include <string.h>

enum { NODE_MAX = 512, NODE_MIN = 16 };

static int reserve(dn_nodes* b, size_t need)
{
	if (need <= b->cap) return 1;
	size_t nc = b->cap ? b->cap : 64;
	while (nc < need) nc *= 2;
	dn_node* nv = (dn_node*)DN_REALLOC(b->v, nc * sizeof(dn_node));
	if (!nv) return 0;
	b->v = nv;
	b->cap = nc;
	return 1;
}

int dn_nodes_init(dn_nodes* b, uint64_t numChunks)
{
	memset(b, 0, sizeof(*b));
	b->voxelCap = (uint64_t)NODE_MAX * numChunks / 2;
	size_t n = (size_t)(b->voxelCap / NODE_MAX);
	if (!reserve(b, n ? n : 1)) return 0;
	for (size_t i = 0; i < n; i++) b->v[i] = (dn_node){NODE_MAX, (uint64_t)i * NODE_MAX, -1};
	b->n = n;
	return 1;
}

void dn_nodes_free(dn_nodes* b)
{
	DN_FREE(b->v);
	memset(b, 0, sizeof(*b));
}

int dn_nodes_grow(dn_nodes* b, uint64_t num)
{
	if (num <= b->voxelCap) return 1;
	/* whole nodes only: a remainder below 512 voxels adds capacity but no node (voxel.c:1064-1077) */
	size_t add = (size_t)((num - b->voxelCap) / NODE_MAX);
	if (!reserve(b, b->n + add)) return 0;
	for (size_t k = 0; k < add; k++) b->v[b->n + k] = (dn_node){NODE_MAX, b->voxelCap + (uint64_t)k * NODE_MAX, -1};
	b->n += add;
	b->voxelCap = num;
	return 1;
}

void dn_nodes_unload(dn_nodes* b, int64_t tile)
{
	for (size_t i = 0; i < b->n; i++)
		if (b->v[i].tile == tile) { b->v[i].tile = -1; return; }
}

int dn_nodes_stream(dn_nodes* b, int64_t tile, uint32_t nvox, const uint32_t* lastUsed, int64_t* victim)
{
	*victim = -1;
	uint32_t need = NODE_MIN;
	while (need < nvox) need <<= 1;
	/* One pass in buffer order.  A free node counts as unused for UINT32_MAX syncs, so it beats every
	 * owned node; among free nodes the smaller one wins, among owned nodes the one unused longer, and
	 * the first found keeps a tie.  A free node of exactly the needed size ends the pass. */
	size_t best = (size_t)-1;
	uint32_t bestTime = 0, bestSize = UINT32_MAX;
	for (size_t i = 0; i < b->n; i++) {
		const dn_node* nd = &b->v[i];
		if (nd->size < need) continue;
		const uint32_t t = nd->tile >= 0 ? lastUsed[nd->tile] : UINT32_MAX;
		if (t > bestTime || (t == UINT32_MAX && nd->size < bestSize)) {
			bestTime = t;
			bestSize = nd->size;
			best = i;
		}
		if (bestSize == need && bestTime == UINT32_MAX) break;
	}
	/* no node, or only chunks used in the last sync: the chunk stays unloaded and the buffer grows */
	if (best == (size_t)-1 || bestTime <= 1) return 0;
	*victim = b->v[best].tile;
	if (bestSize > need) {
		/* split: [need][need][2 need][4 need]... covering the old node */
		size_t extra = 0;
		for (uint32_t s = bestSize; s > need; s >>= 1) extra++;
		if (!reserve(b, b->n + extra)) return -1;
		memmove(&b->v[best + 1 + extra], &b->v[best + 1], (b->n - best - 1) * sizeof(dn_node));
		const uint64_t org = b->v[best].start;
		b->v[best] = (dn_node){need, org, -1};
		uint32_t s = need;
		for (size_t k = 1; k <= extra; k++, s <<= 1) b->v[best + k] = (dn_node){s, org + s, -1};
		b->n += extra;
	}
	b->v[best].tile = tile;
	return 1;
}

void dn_nodes_sort(dn_nodes* b, int maxCopies)
{
	/* one bubble pass towards: owned nodes first, then free nodes by descending size; adjacent equal
	 * free nodes below 512 merge.  Each swap or merge counts as one copy. */
	int copies = 0;
	for (size_t i = 0; i + 1 < b->n; i++) {
		dn_node cur = b->v[i], nxt = b->v[i + 1];
		if (cur.tile >= 0) continue;
		if (nxt.tile >= 0 || nxt.size < cur.size) {
			copies++;
			nxt.start -= cur.size;
			cur.start += nxt.size;
			b->v[i] = nxt;
			b->v[i + 1] = cur;
		}
		if (nxt.tile < 0 && cur.size == nxt.size && cur.size < NODE_MAX) {
			copies++;
			b->v[i].size *= 2;
			memmove(&b->v[i + 1], &b->v[i + 2], (b->n - i - 2) * sizeof(dn_node));
			b->n--;
		}
		if (copies > maxCopies) break;
	}
}
