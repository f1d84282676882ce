/*
 * serve.h -- a request loop over many resident volumes (addition; the reference has no serving layer: its
 * application renders one volume per GL context from its own frame loop, main.c:449-520).
 *
 * Requests arrive from any thread (DN_server_submit) and are served by the server's own thread in ticks.
 * Each tick is one batched frame (DN_batch_run) over the volumes that have queued work, so requests that
 * arrive while earlier ticks are on the GPU are admitted into the next tick and run beside the other
 * volumes' requests.  A volume's requests run in arrival order, and each kind is a fixed sequence of the
 * reference's calls:
 *   draw     DN_draw(vol, output, view, projection, rasterColorTexture, rasterDepthTexture)
 *   relight  DN_sync_gpu(vol, DN_READ_WRITE, 1) then DN_update_lighting(vol, numDiffuse, maxDiffuse, time)
 *   edit     the voxel edits on the CPU map (DN_set_voxel / DN_remove_voxel), then DN_sync_gpu(vol,
 *            DN_READ_WRITE, 1): changed chunks are re-staged in place and their lighting history reset
 * so a volume's results do not depend on which other requests share its ticks.
 *
 * Admission: a tick only includes volumes whose device state fits the device budget together with every
 * other resident volume; when it does not fit, the least recently used idle volumes are evicted whole to
 * pinned host memory (dn_cuda_map_evict) and restored on their next request.  Evictions and restores are
 * queued in the batch's stream order (no host wait); their copies count in the tick's device time.
 */
#ifndef DN_SERVE_H
#define DN_SERVE_H

#include "voxel.h"

#ifdef __cplusplus
extern "C"
{
#endif

typedef struct DNserver DNserver;

typedef enum DNrequestKind
{
	DN_REQUEST_DRAW = 0,
	DN_REQUEST_RELIGHT = 1,
	DN_REQUEST_EDIT = 2
} DNrequestKind;

typedef struct DNvoxelEdit
{
	DNivec3 mapPos, chunkPos;
	DNvoxel voxel;
	int remove;                      /* 1: DN_remove_voxel instead of DN_set_voxel */
} DNvoxelEdit;

typedef struct DNrequest
{
	DNrequestKind kind;
	unsigned int volume;             /* index returned by DN_server_add_volume */
	DNimage* output;                 /* draw: written when the request completes */
	DNmat4 view, projection;
	int numDiffuseSamples, maxDiffuseSamples;   /* relight */
	float time;
	const DNvoxelEdit* edits;        /* edit: copied at submission */
	unsigned int numEdits;
	void* user;                      /* returned with the completion */
	int rasterColorTexture, rasterDepthTexture;   /* draw: as DN_draw (0: none) */
} DNrequest;

typedef struct DNcompletion
{
	uint64_t id;
	void* user;
	DNrequestKind kind;
	unsigned int volume;
	double arrival, admitted, finished;   /* seconds on the server's monotonic clock */
	int ok;
} DNcompletion;

typedef struct DNserveConfig
{
	uint64_t deviceBudgetBytes;      /* 0: no limit */
	unsigned int maxVolumesPerTick;  /* 0: no limit */
	unsigned int maxTicksInFlight;   /* 1 or 2 (0 means 2) */
} DNserveConfig;

typedef struct DNserveStats
{
	uint64_t submitted, completed, failed;
	uint64_t ticks, items;
	uint64_t evictions, restores;
	uint64_t residentBytes;
	unsigned int residentVolumes;
	/* where the time goes: the serving thread's residency decisions (evictions and restores issued) and
	 * tick issue (DN_batch_run), the device time of retired ticks (restore / evict copies included), and
	 * the bytes evicted and restored */
	double admitSeconds, issueSeconds, deviceSeconds;
	uint64_t evictedBytes, restoredBytes;
	double evictSeconds, restoreSeconds;     /* the serving thread's time inside dn_cuda_map_evict / _restore */
} DNserveStats;

DNserver* DN_server_create(const DNserveConfig* config);
/* stops the serving thread and frees the server: ticks in flight finish, requests still queued are
 * dropped (call DN_server_drain first to serve them); the volumes stay the caller's, resident */
void DN_server_destroy(DNserver* server);
/* registers a device volume (it joins the server's batch); returns its index, or -1 */
int DN_server_add_volume(DNserver* server, DNvolume* vol);
/* starts the serving thread.  When the volumes' device footprint exceeds the budget, the pinned host memory
 * their evictions need (the excess plus a quarter) is reserved here (dn_cuda_host_reserve), so that no
 * eviction under load pins host memory, and volumes are evicted down to the budget (least recently used
 * first; volumes not used yet in the order they were added) before the thread takes requests; false if the
 * reservation or an eviction fails */
bool DN_server_start(DNserver* server);
/* thread-safe; returns the request id (> 0), or 0 for an invalid request */
uint64_t DN_server_submit(DNserver* server, const DNrequest* request);
/* submits requests[i] at offsets[i] seconds after the call (non-decreasing) from the calling thread */
size_t DN_server_replay(DNserver* server, const DNrequest* requests, const double* offsets, size_t count);
/* waits until every submitted request has completed and the serving thread is idle with its resident set
 * within the budget: volumes grow when their syncs stage chunks, and the idle thread evicts (least recently
 * used first) down to the budget before it waits for more work (false on timeout) */
bool DN_server_drain(DNserver* server, double timeoutSeconds);
/* moves up to capacity completions out of the server; returns how many */
size_t DN_server_poll(DNserver* server, DNcompletion* out, size_t capacity);
void DN_server_get_stats(DNserver* server, DNserveStats* out);
/* the batch the server runs its ticks on (counters, tuning) */
DNbatch* DN_server_batch(DNserver* server);
/* seconds on the server's monotonic clock */
double DN_server_clock(void);

#ifdef __cplusplus
}
#endif

#endif
