/*
 * dn_serve.c -- the request loop of include/DoonEngine/serve.h.
 *
 * One serving thread owns the GPU side: it sorts arrivals into per-volume FIFOs, builds a tick from the
 * volumes with queued work (oldest head request first), restores or evicts volumes to keep the resident
 * set under the device budget, launches the tick as one batched frame and records an event after it.
 * Up to two ticks are in flight, so the host builds tick n+1 while the GPU runs tick n.  A request
 * completes when the event of its tick has fired.
 *
 * A tick takes, from each volume's FIFO, the longest prefix that fits one batched item, whose phases run
 * in the order draw, sync, lighting: at most one draw, then at most one sync-bearing request (an edit, or
 * a relight which also lights).  Each request kind maps to a fixed sequence of the reference's calls, so
 * the volume sees the same sequence however its requests are grouped into ticks.
 */
#include "DoonEngine/serve.h"
#include "dn_cuda.h"
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct Pending
{
	uint64_t id;
	DNrequest req;
	DNvoxelEdit* edits;              /* owned copy of req.edits */
	double arrival, admitted;
	struct Pending* next;
} Pending;

typedef struct VolumeSlot
{
	DNvolume* vol;
	Pending* head;
	Pending* tail;
	uint64_t lastTick;               /* last tick that used the volume (LRU) */
	unsigned int inFlight;           /* ticks in flight that use the volume */
	int resident;
	int restoring;                   /* resident, its restore copies possibly still running */
} VolumeSlot;

typedef struct Tick
{
	void* event;
	void* started;          /* recorded before the tick's evictions, restores and launches */
	Pending** reqs;
	size_t nreqs, cap;
	unsigned int* vols;
	size_t nvols, volsCap;
} Tick;

struct DNserver
{
	DNserveConfig cfg;
	DNbatch* batch;
	VolumeSlot* slots;
	unsigned int nslots;
	size_t slotsCap;
	pthread_mutex_t lock;
	pthread_cond_t cond;
	Pending* inHead;
	Pending* inTail;
	uint64_t nextId;
	uint64_t outstanding;            /* submitted and not yet completed */
	DNcompletion* done;
	size_t ndone, doneCap;
	pthread_t thread;
	int started, stop;
	int cancel;                      /* stop serving queued requests: they complete with ok = 0 */
	int settled;                     /* the thread is idle with the resident set within the budget */
	Tick ticks[2];
	unsigned int tickHead, tickCount;
	uint64_t tickNo;
	DNserveStats stats;
	DNbatchItem* items;
	size_t itemsCap;
	unsigned int* order;
	size_t orderCap;
};

double DN_server_clock(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void sleep_us(long us)
{
	struct timespec ts = {us / 1000000, (us % 1000000) * 1000};
	nanosleep(&ts, NULL);
}

static bool grow(void** p, size_t* cap, size_t need, size_t elem)
{
	if (need <= *cap) return true;
	size_t nc = *cap ? *cap : 16;
	while (nc < need) nc *= 2;
	void* np = realloc(*p, nc * elem);
	if (!np) return false;
	*p = np;
	*cap = nc;
	return true;
}

DNserver* DN_server_create(const DNserveConfig* cfg)
{
	DNserver* s = (DNserver*)calloc(1, sizeof(DNserver));
	if (!s) return NULL;
	if (cfg) s->cfg = *cfg;
	if (s->cfg.maxTicksInFlight == 0 || s->cfg.maxTicksInFlight > 2) s->cfg.maxTicksInFlight = 2;
	s->batch = DN_batch_create();
	if (!s->batch) { free(s); return NULL; }
	for (int i = 0; i < 2; i++)
		if (dn_cuda_event_create(&s->ticks[i].event) != DN_CUDA_OK ||
		    dn_cuda_event_create(&s->ticks[i].started) != DN_CUDA_OK) {
			DN_batch_destroy(s->batch);
			free(s);
			return NULL;
		}
	pthread_mutex_init(&s->lock, NULL);
	pthread_cond_init(&s->cond, NULL);
	s->nextId = 1;
	return s;
}

int DN_server_add_volume(DNserver* s, DNvolume* vol)
{
	if (!s || !vol || s->started) return -1;
	if (!grow((void**)&s->slots, &s->slotsCap, (size_t)s->nslots + 1, sizeof(VolumeSlot))) return -1;
	if (!DN_batch_add(s->batch, vol)) return -1;
	VolumeSlot* v = &s->slots[s->nslots];
	memset(v, 0, sizeof(*v));
	v->vol = vol;
	v->resident = dn_cuda_map_is_resident(vol->gpu);
	return (int)s->nslots++;
}

static void free_pending(Pending* p)
{
	free(p->edits);
	free(p);
}

uint64_t DN_server_submit(DNserver* s, const DNrequest* r)
{
	if (!s || !r || r->volume >= s->nslots) return 0;
	if (r->kind == DN_REQUEST_DRAW && (!r->output || !r->output->color || !r->output->width || !r->output->height)) return 0;
	if (r->kind == DN_REQUEST_EDIT && r->numEdits && !r->edits) return 0;
	/* a draw composed with raster textures names one texture of each kind (as DN_draw checks) */
	if (r->kind == DN_REQUEST_DRAW && r->rasterColorTexture > 0 && r->rasterDepthTexture > 0 &&
	    (DN_texture_format(r->rasterColorTexture) != DN_TEXTURE_RGBA32F ||
	     DN_texture_format(r->rasterDepthTexture) != DN_TEXTURE_DEPTH32F)) return 0;
	if (r->kind > DN_REQUEST_EDIT) return 0;
	Pending* p = (Pending*)calloc(1, sizeof(Pending));
	if (!p) return 0;
	p->req = *r;
	if (r->kind == DN_REQUEST_EDIT && r->numEdits) {
		p->edits = (DNvoxelEdit*)malloc(sizeof(DNvoxelEdit) * r->numEdits);
		if (!p->edits) { free(p); return 0; }
		memcpy(p->edits, r->edits, sizeof(DNvoxelEdit) * r->numEdits);
	}
	p->req.edits = p->edits;
	p->arrival = DN_server_clock();
	pthread_mutex_lock(&s->lock);
	p->id = s->nextId++;
	if (s->inTail) s->inTail->next = p; else s->inHead = p;
	s->inTail = p;
	s->outstanding++;
	s->stats.submitted++;
	s->settled = 0;
	pthread_cond_signal(&s->cond);
	pthread_mutex_unlock(&s->lock);
	return p->id;
}

size_t DN_server_replay(DNserver* s, const DNrequest* reqs, const double* offsets, size_t n)
{
	const double t0 = DN_server_clock();
	size_t k = 0;
	for (size_t i = 0; i < n; i++) {
		for (;;) {
			const double wait = t0 + offsets[i] - DN_server_clock();
			if (wait <= 0.0) break;
			if (wait > 300e-6) sleep_us((long)((wait - 200e-6) * 1e6));
		}
		if (DN_server_submit(s, &reqs[i])) k++;
	}
	return k;
}

/* ------------------------------------------------------------ residency */

static uint64_t resident_bytes(DNserver* s, unsigned int* count)
{
	uint64_t b = 0;
	unsigned int n = 0;
	for (unsigned int i = 0; i < s->nslots; i++)
		if (s->slots[i].resident) { b += dn_cuda_map_footprint(s->slots[i].vol->gpu); n++; }
	if (count) *count = n;
	return b;
}

/* evicts idle least-recently-used volumes (not in the tick being built, inTick[i] != 0, and not in a
 * tick in flight) until the resident set plus extra bytes fits the budget; false if it cannot */
static bool enforce_budget(DNserver* s, uint64_t extra, const uint8_t* inTick)
{
	const uint64_t budget = s->cfg.deviceBudgetBytes;
	if (!budget) return true;
	uint64_t used = resident_bytes(s, NULL);
	while (used + extra > budget) {
		int victim = -1;
		for (unsigned int i = 0; i < s->nslots; i++) {
			VolumeSlot* c = &s->slots[i];
			if (!c->resident || c->inFlight || c->restoring || (inTick && inTick[i])) continue;
			if (victim < 0 || c->lastTick < s->slots[victim].lastTick) victim = (int)i;
		}
		if (victim < 0) return false;
		const uint64_t bytes = dn_cuda_map_footprint(s->slots[victim].vol->gpu);
		const double e0 = DN_server_clock();
		if (dn_cuda_map_evict(s->slots[victim].vol->gpu) != DN_CUDA_OK) return false;
		s->stats.evictSeconds += DN_server_clock() - e0;
		s->slots[victim].resident = 0;
		s->stats.evictions++;
		s->stats.evictedBytes += bytes;
		used = resident_bytes(s, NULL);
	}
	return true;
}

/* true when volume v can join the tick being built: resident with its restore copies done.  An evicted
 * volume is restored within the budget without any stream waiting for it (dn_cuda_map_restore_async), and
 * joins a later tick once the copies are done, so the other volumes' requests never wait for them.  False
 * also when the budget cannot make room now; a volume larger than the whole budget still runs once nothing
 * else is resident. */
static bool admit(DNserver* s, unsigned int v, const uint8_t* inTick)
{
	VolumeSlot* slot = &s->slots[v];
	if (slot->resident) {
		if (!slot->restoring) return true;
		if (dn_cuda_map_restore_query(slot->vol->gpu) == 0) return false;
		slot->restoring = 0;   /* done (an error shows at the volume's next use) */
		return true;
	}
	if (!enforce_budget(s, dn_cuda_map_footprint(slot->vol->gpu), inTick)) {
		unsigned int n = 0;
		resident_bytes(s, &n);
		if (n) return false;
	}
	const double r0 = DN_server_clock();
	if (dn_cuda_map_restore_async(slot->vol->gpu) != DN_CUDA_OK) return false;
	s->stats.restoreSeconds += DN_server_clock() - r0;
	slot->resident = 1;
	slot->restoring = 1;
	s->stats.restores++;
	s->stats.restoredBytes += dn_cuda_map_footprint(slot->vol->gpu);
	return false;
}

static bool any_restoring(const DNserver* s)
{
	for (unsigned int i = 0; i < s->nslots; i++)
		if (s->slots[i].restoring) return true;
	return false;
}

/* ----------------------------------------------------------------- ticks */

static void apply_edits(DNvolume* vol, const Pending* p)
{
	for (unsigned int e = 0; e < p->req.numEdits; e++) {
		const DNvoxelEdit* ed = &p->edits[e];
		if (!DN_in_map_bounds(vol, ed->mapPos) || !DN_in_chunk_bounds(ed->chunkPos)) continue;
		if (ed->remove) DN_remove_voxel(vol, ed->mapPos, ed->chunkPos);
		else DN_set_voxel(vol, ed->mapPos, ed->chunkPos, ed->voxel);
	}
}

static int cmp_head(const void* a, const void* b, void* ctx)
{
	const DNserver* s = (const DNserver*)ctx;
	const double x = s->slots[*(const unsigned int*)a].head->arrival;
	const double y = s->slots[*(const unsigned int*)b].head->arrival;
	return x < y ? -1 : (x > y ? 1 : 0);
}

/* insertion sort by head arrival (the candidate list is short and mostly ordered already) */
static void sort_candidates(DNserver* s, unsigned int* v, size_t n)
{
	for (size_t i = 1; i < n; i++) {
		unsigned int x = v[i];
		size_t j = i;
		while (j > 0 && cmp_head(&v[j - 1], &x, s) > 0) { v[j] = v[j - 1]; j--; }
		v[j] = x;
	}
}

/* builds and launches one tick; returns 1 when a tick was launched, 0 when there was nothing to run,
 * -1 on a launch failure (its requests complete with ok = 0) */
static int launch_tick(DNserver* s)
{
	size_t nc = 0;
	for (unsigned int i = 0; i < s->nslots; i++) if (s->slots[i].head) nc++;
	if (!nc) return 0;
	if (!grow((void**)&s->order, &s->orderCap, nc, sizeof(unsigned int))) return 0;
	nc = 0;
	for (unsigned int i = 0; i < s->nslots; i++) if (s->slots[i].head) s->order[nc++] = i;
	sort_candidates(s, s->order, nc);
	uint8_t* inTick = (uint8_t*)calloc(s->nslots, 1);
	if (!inTick) return 0;
	Tick* t = &s->ticks[(s->tickHead + s->tickCount) % 2];
	const double t0 = DN_server_clock();
	dn_cuda_event_record(t->started, DN_batch_stream(s->batch));
	/* volumes grow as they stage chunks: bring the resident set back under the budget first */
	enforce_budget(s, 0, inTick);
	t->nreqs = 0;
	t->nvols = 0;
	size_t nitems = 0;
	const double now = DN_server_clock();
	const unsigned int maxVols = s->cfg.maxVolumesPerTick ? s->cfg.maxVolumesPerTick : 0xFFFFFFFFu;
	for (size_t c = 0; c < nc && nitems < maxVols; c++) {
		const unsigned int v = s->order[c];
		VolumeSlot* slot = &s->slots[v];
		if (!admit(s, v, inTick)) continue;
		if (!grow((void**)&s->items, &s->itemsCap, nitems + 1, sizeof(DNbatchItem)) ||
		    !grow((void**)&t->vols, &t->volsCap, t->nvols + 1, sizeof(unsigned int)))
			break;
		DNbatchItem* it = &s->items[nitems];
		memset(it, 0, sizeof(*it));
		it->vol = slot->vol;
		int pos = 0;       /* 1 after a draw, 2 after a sync, 3 after lighting */
		while (slot->head) {
			Pending* p = slot->head;
			const DNrequest* r = &p->req;
			if (r->kind == DN_REQUEST_DRAW) {
				if (pos >= 1) break;
				it->phases |= DN_PHASE_DRAW;
				it->output = r->output; it->view = r->view; it->projection = r->projection;
				it->rasterColorTexture = r->rasterColorTexture; it->rasterDepthTexture = r->rasterDepthTexture;
				pos = 1;
			} else {
				if (pos >= 2) break;
				it->phases |= DN_PHASE_SYNC;
				it->op = DN_READ_WRITE;
				it->lightingSplit = 1;
				if (r->kind == DN_REQUEST_EDIT) {
					apply_edits(slot->vol, p);
					pos = 2;
				} else {
					it->phases |= DN_PHASE_LIGHT;
					it->numDiffuseSamples = r->numDiffuseSamples;
					it->maxDiffuseSamples = r->maxDiffuseSamples;
					it->time = r->time;
					pos = 3;
				}
			}
			if (!grow((void**)&t->reqs, &t->cap, t->nreqs + 1, sizeof(Pending*))) break;
			slot->head = p->next;
			if (!slot->head) slot->tail = NULL;
			p->next = NULL;
			p->admitted = now;
			t->reqs[t->nreqs++] = p;
		}
		if (!it->phases) continue;
		inTick[v] = 1;
		slot->lastTick = s->tickNo;
		slot->inFlight++;
		t->vols[t->nvols++] = v;
		nitems++;
	}
	free(inTick);
	const double t1 = DN_server_clock();
	s->stats.admitSeconds += t1 - t0;
	if (!nitems) {
		/* nothing ran; the start event may have been recorded: close the (empty) interval */
		dn_cuda_event_record(t->event, DN_batch_stream(s->batch));
		return 0;
	}
	s->tickNo++;
	s->stats.ticks++;
	s->stats.items += nitems;
	int ok = DN_batch_run(s->batch, s->items, (unsigned int)nitems) ? 1 : 0;
	if (ok && dn_cuda_event_record(t->event, DN_batch_stream(s->batch)) != DN_CUDA_OK) ok = 0;
	s->stats.issueSeconds += DN_server_clock() - t1;
	s->tickCount++;
	if (!ok) {
		/* the tick's requests fail; make the event fire now so the completion path retires them */
		for (size_t i = 0; i < t->nreqs; i++) t->reqs[i]->admitted = -1.0;
		DN_batch_finish(s->batch);
		dn_cuda_event_record(t->event, DN_batch_stream(s->batch));
		return -1;
	}
	return 1;
}

/* retires the oldest tick if its event fired (block: wait for it); returns 1 when a tick was retired */
static int retire_tick(DNserver* s, int block)
{
	if (!s->tickCount) return 0;
	Tick* t = &s->ticks[s->tickHead];
	if (block) {
		while (dn_cuda_event_query(t->event) == 0) sleep_us(20);
	} else if (dn_cuda_event_query(t->event) == 0) {
		return 0;
	}
	const double now = DN_server_clock();
	float ms = 0.0f;
	if (dn_cuda_event_elapsed_ms(t->started, t->event, &ms) == DN_CUDA_OK) s->stats.deviceSeconds += ms * 1e-3;
	pthread_mutex_lock(&s->lock);
	if (grow((void**)&s->done, &s->doneCap, s->ndone + t->nreqs, sizeof(DNcompletion))) {
		for (size_t i = 0; i < t->nreqs; i++) {
			const Pending* p = t->reqs[i];
			DNcompletion* c = &s->done[s->ndone++];
			c->id = p->id; c->user = p->req.user; c->kind = p->req.kind; c->volume = p->req.volume;
			c->arrival = p->arrival; c->admitted = p->admitted; c->finished = now;
			c->ok = p->admitted >= 0.0;
			if (!c->ok) s->stats.failed++;
		}
	}
	s->stats.completed += t->nreqs;
	s->outstanding -= t->nreqs;
	pthread_cond_broadcast(&s->cond);
	pthread_mutex_unlock(&s->lock);
	for (size_t i = 0; i < t->nreqs; i++) free_pending(t->reqs[i]);
	t->nreqs = 0;
	for (size_t i = 0; i < t->nvols; i++) s->slots[t->vols[i]].inFlight--;
	t->nvols = 0;
	s->tickHead = (s->tickHead + 1) % 2;
	s->tickCount--;
	return 1;
}

static void* serve_main(void* arg)
{
	DNserver* s = (DNserver*)arg;
	for (;;) {
		pthread_mutex_lock(&s->lock);
		Pending* in = s->inHead;
		s->inHead = s->inTail = NULL;
		const int stop = s->stop;
		pthread_mutex_unlock(&s->lock);
		while (in) {
			Pending* next = in->next;
			in->next = NULL;
			VolumeSlot* slot = &s->slots[in->req.volume];
			if (slot->tail) slot->tail->next = in; else slot->head = in;
			slot->tail = in;
			in = next;
		}
		if (s->cancel) {
			/* queued requests are not served any more: complete them as failed */
			pthread_mutex_lock(&s->lock);
			for (unsigned int i = 0; i < s->nslots; i++) {
				for (Pending* p = s->slots[i].head; p;) {
					Pending* n = p->next;
					if (grow((void**)&s->done, &s->doneCap, s->ndone + 1, sizeof(DNcompletion))) {
						DNcompletion* c = &s->done[s->ndone++];
						c->id = p->id; c->user = p->req.user; c->kind = p->req.kind; c->volume = p->req.volume;
						c->arrival = p->arrival; c->admitted = -1.0; c->finished = DN_server_clock(); c->ok = 0;
					}
					s->stats.completed++;
					s->stats.failed++;
					s->outstanding--;
					free_pending(p);
					p = n;
				}
				s->slots[i].head = s->slots[i].tail = NULL;
			}
			pthread_cond_broadcast(&s->cond);
			pthread_mutex_unlock(&s->lock);
		}
		int progressed = 0;
		if (s->tickCount < s->cfg.maxTicksInFlight && launch_tick(s) != 0) progressed = 1;
		if (retire_tick(s, s->tickCount >= s->cfg.maxTicksInFlight)) progressed = 1;
		if (progressed) continue;
		int queued = 0;
		for (unsigned int i = 0; i < s->nslots && !queued; i++) queued = s->slots[i].head != NULL;
		if (stop && !queued && !s->tickCount) break;
		if (s->tickCount || (queued && any_restoring(s))) {
			/* the GPU is busy: pin one more slab if fewer are free than in use (evictions under load then
			 * find them pinned; volumes keep growing as their chunks stream in, so the evicted set does) */
			if (s->cfg.deviceBudgetBytes) {
				const uint64_t pinned = dn_cuda_host_pinned(), spare = dn_cuda_host_pinned_free();
				if (pinned - spare > spare && dn_cuda_host_headroom(spare + dn_cuda_host_slab_bytes()) == DN_CUDA_OK)
					continue;
			}
			sleep_us(20);
			continue;
		}
		if (!queued && !s->settled) {
			/* idle: volumes grow when their syncs stage chunks, so a busy period can end above the budget;
			 * evict down to it now, while no request waits (DN_server_drain waits for this too) */
			enforce_budget(s, 0, NULL);
			if (s->cfg.deviceBudgetBytes) {
				/* which maps are evicted changes under load, and small maps round up to whole slabs: keep as
				 * much pinned memory free as is in use, pinned now rather than by an eviction in a tick
				 * (pinning a 64 MiB slab takes milliseconds, and the serving thread would hold every request
				 * for it; measured, a quarter and a half of it still left slabs to pin under load) */
				const uint64_t pinned = dn_cuda_host_pinned(), spare = dn_cuda_host_pinned_free();
				if (pinned > spare) dn_cuda_host_headroom(pinned - spare);
			}
			pthread_mutex_lock(&s->lock);
			if (!s->inHead) s->settled = 1;
			pthread_cond_broadcast(&s->cond);
			pthread_mutex_unlock(&s->lock);
			continue;
		}
		/* idle: wait for a submission */
		pthread_mutex_lock(&s->lock);
		if (!s->inHead && !s->stop) {
			struct timespec ts;
			clock_gettime(CLOCK_REALTIME, &ts);
			ts.tv_nsec += 2000000;
			if (ts.tv_nsec >= 1000000000) { ts.tv_sec++; ts.tv_nsec -= 1000000000; }
			pthread_cond_timedwait(&s->cond, &s->lock, &ts);
		}
		pthread_mutex_unlock(&s->lock);
	}
	pthread_mutex_lock(&s->lock);
	s->settled = 1;
	pthread_cond_broadcast(&s->cond);
	pthread_mutex_unlock(&s->lock);
	return NULL;
}

bool DN_server_start(DNserver* s)
{
	if (!s || s->started) return false;
	/* volumes beyond the budget will be evicted: pin the host memory they need now, not under load (the
	 * difference plus a quarter, for growth and slab rounding) */
	if (s->cfg.deviceBudgetBytes) {
		const uint64_t used = resident_bytes(s, NULL);
		if (used > s->cfg.deviceBudgetBytes) {
			const uint64_t over = used - s->cfg.deviceBudgetBytes;
			if (dn_cuda_host_reserve(over + over / 4) != DN_CUDA_OK) return false;
			/* and evict down to the budget before the first request arrives, so that no request waits on
			 * the start's evictions (counted in the stats like any other) */
			if (!enforce_budget(s, 0, NULL)) return false;
		}
	}
	s->stop = 0;
	if (pthread_create(&s->thread, NULL, serve_main, s) != 0) return false;
	s->started = 1;
	return true;
}

bool DN_server_drain(DNserver* s, double timeout)
{
	if (!s) return false;
	const double end = DN_server_clock() + timeout;
	pthread_mutex_lock(&s->lock);
	while (s->outstanding || (s->started && !s->settled)) {
		if (DN_server_clock() > end) { pthread_mutex_unlock(&s->lock); return false; }
		struct timespec ts;
		clock_gettime(CLOCK_REALTIME, &ts);
		ts.tv_nsec += 1000000;
		if (ts.tv_nsec >= 1000000000) { ts.tv_sec++; ts.tv_nsec -= 1000000000; }
		pthread_cond_timedwait(&s->cond, &s->lock, &ts);
	}
	pthread_mutex_unlock(&s->lock);
	return true;
}

size_t DN_server_poll(DNserver* s, DNcompletion* out, size_t cap)
{
	if (!s) return 0;
	pthread_mutex_lock(&s->lock);
	size_t n = s->ndone < cap ? s->ndone : cap;
	if (n) {
		memcpy(out, s->done, n * sizeof(DNcompletion));
		memmove(s->done, s->done + n, (s->ndone - n) * sizeof(DNcompletion));
		s->ndone -= n;
	}
	pthread_mutex_unlock(&s->lock);
	return n;
}

void DN_server_get_stats(DNserver* s, DNserveStats* out)
{
	if (!s || !out) return;
	pthread_mutex_lock(&s->lock);
	*out = s->stats;
	pthread_mutex_unlock(&s->lock);
	out->residentBytes = resident_bytes(s, &out->residentVolumes);
}

DNbatch* DN_server_batch(DNserver* s) { return s ? s->batch : NULL; }

void DN_server_destroy(DNserver* s)
{
	if (!s) return;
	if (s->started) {
		pthread_mutex_lock(&s->lock);
		s->stop = 1;
		s->cancel = 1;
		pthread_cond_broadcast(&s->cond);
		pthread_mutex_unlock(&s->lock);
		pthread_join(s->thread, NULL);
	}
	DN_batch_finish(s->batch);
	for (Pending* p = s->inHead; p;) { Pending* n = p->next; free_pending(p); p = n; }
	for (unsigned int i = 0; i < s->nslots; i++)
		for (Pending* p = s->slots[i].head; p;) { Pending* n = p->next; free_pending(p); p = n; }
	for (int i = 0; i < 2; i++) {
		for (size_t k = 0; k < s->ticks[i].nreqs; k++) free_pending(s->ticks[i].reqs[k]);
		free(s->ticks[i].reqs);
		free(s->ticks[i].vols);
		dn_cuda_event_destroy(s->ticks[i].event);
		dn_cuda_event_destroy(s->ticks[i].started);
	}
	for (unsigned int i = 0; i < s->nslots; i++) {
		/* volumes go back to the caller resident and out of the server's batch */
		if (!s->slots[i].resident || s->slots[i].restoring) dn_cuda_map_restore(s->slots[i].vol->gpu);
		s->slots[i].restoring = 0;
		DN_batch_remove(s->batch, s->slots[i].vol);
	}
	DN_batch_destroy(s->batch);
	pthread_mutex_destroy(&s->lock);
	pthread_cond_destroy(&s->cond);
	free(s->slots);
	free(s->done);
	free(s->items);
	free(s->order);
	free(s);
}
