/*
 * dn_shapes.cu -- the signed-distance pass of the shape functions (src/DoonEngine/voxelShapes.c) on the
 * device: dn_cuda_shape_eval of include/dn_cuda.h.
 *
 * The reference walks every voxel of every chunk a shape's bounding box covers on the CPU, evaluates the
 * shape's distance at the voxel (after the inverse transform) and, for voxels it edits, a forward-
 * difference normal from three more distance evaluations (voxelShapes.c:131-147, 183-232; the sphere
 * uses the squared distance to its centre instead, 246-337).  Here one block of 512 threads takes one
 * chunk, a thread per voxel, and the edits come back as a compact list in the reference's visiting order:
 *   pass 1 (k_shape_count): each chunk's number of edited voxels;
 *   host:                   exclusive prefix over the chunks;
 *   pass 2 (k_shape_write): each edited voxel's record at its chunk's offset plus its rank among the
 *                           chunk's edited voxels in voxel order z, y, x (warp ballots + a block scan).
 * The host side (voxelShapes.c of this library) applies the list to the CPU map with the reference's
 * rules.  Every float operation is the reference's, in its order, with no contraction, so the distances
 * and normals are bit-identical to the reference's x86 build.  Where the reference passes floats through
 * double fmin / fmax / fabs or multiplies two of them in double, the single-precision operation gives the
 * same float (a min / max returns one of its operands; the product of two floats is exact in double and
 * is rounded once either way); only the cylinder's two double sums stay in double.
 */
#include "dn_internal.cuh"
#include <stdlib.h>
#include <string.h>

namespace {

struct V3 { float x, y, z; };

// m * (x, y, z, w) for a column-major matrix: ((c0 x + c1 y) + c2 z) + c3 w per component, the order of
// the reference's SSE column product (quickmath.h:206-216)
__device__ __forceinline__ V3 xform(const float (*m)[4], float x, float y, float z, float w)
{
    V3 r;
    r.x = m[0][0] * x + m[1][0] * y + m[2][0] * z + m[3][0] * w;
    r.y = m[0][1] * x + m[1][1] * y + m[2][1] * z + m[3][1] * w;
    r.z = m[0][2] * x + m[1][2] * y + m[2][2] * z + m[3][2] * w;
    return r;
}

__device__ __forceinline__ float len2(float x, float y) { return sqrtf(x * x + y * y); }
__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }
// the reference's component max (a > b ? a : b)
__device__ __forceinline__ float gt_max(float a, float b) { return a > b ? a : b; }

// distance functions of voxelShapes.c:23-89, evaluated in shape space
__device__ float shape_sdf(const dn_shape_params& p, V3 q)
{
    switch (p.kind) {
    case DN_SHAPE_BOX:
    case DN_SHAPE_ROUNDED_BOX: {
        const float ax = fabsf(q.x) - p.length[0], ay = fabsf(q.y) - p.length[1], az = fabsf(q.z) - p.length[2];
        const float q1 = len3(gt_max(ax, 0.0f), gt_max(ay, 0.0f), gt_max(az, 0.0f));
        const float q2 = fminf(fmaxf(fmaxf(ax, ay), az), 0.0f);
        const float d = q1 + q2;
        return p.kind == DN_SHAPE_BOX ? d : d - p.radius;
    }
    case DN_SHAPE_TORUS: {
        const float a = len2(q.x, q.z) - p.radius;
        return len2(a, q.y) - p.radiusB;
    }
    case DN_SHAPE_ELLIPSOID: {
        const float l = len3(q.x / p.radii[0], q.y / p.radii[1], q.z / p.radii[2]);
        return (l - 1.0f) * fminf(fminf(p.radii[0], p.radii[1]), p.radii[2]);
    }
    case DN_SHAPE_CYLINDER: {
        // the two sums the reference forms in double (a float result rounded once more could differ)
        const float dx = len2(q.x, q.z) - p.radius, dy = (float)(fabs((double)q.y) - (double)p.height);
        const float a = fminf(fmaxf(dx, dy), 0.0f);
        return (float)((double)a + (double)len2(gt_max(dx, 0.0f), gt_max(dy, 0.0f)));
    }
    case DN_SHAPE_CONE: {
        const float l = len2(q.x, q.z);
        const float dt = p.angles[0] * l + p.angles[1] * q.y;
        return fmaxf(dt, -p.height - q.y);
    }
    case DN_SHAPE_PYRAMID: {
        const float h = p.height;
        const float m2 = h * h * 0.25f;
        float px = fabsf(q.x) / p.length[0], pz = fabsf(q.z) / p.length[2];
        const float py = q.y;
        if (pz > px) { const float t = px; px = pz; pz = t; }
        px -= 0.5f;
        pz -= 0.5f;
        const float qx = pz, qy = h * py - 0.5f * px, qz = h * px + 0.5f * py;
        const float s = fmaxf(-qx, 0.0f);
        const float t = fmaxf(fminf((qy - 0.5f * pz) / (m2 + 0.25f), 0.0f), 1.0f);
        const float a = m2 * (qx + s) * (qx + s) + qy * qy;
        const float b = m2 * (qx + 0.5f * t) * (qx + 0.5f * t) + (qy - m2 * t) * (qy - m2 * t);
        const float d2 = fminf(qy, -qx * m2 - qy * 0.5f) > 0.0f ? 0.0f : fminf(a, b);
        return sqrtf((d2 + qz * qz) / m2) * (fmaxf(qz, -py) >= 0.0f ? 1.0f : -1.0f);
    }
    default:
        return 1.0f;
    }
}

// classification of the voxel at integer coordinates (gx, gy, gz): 0 untouched, 1 inside, 2 shell; the
// normal where the reference computes one (inside voxels of a placement, shell voxels), unflipped
__device__ uint32_t shape_classify(const dn_shape_params& p, int gx, int gy, int gz, float n[3])
{
    const float px = (float)gx, py = (float)gy, pz = (float)gz;
    n[0] = n[1] = n[2] = 0.0f;
    if (p.kind == DN_SHAPE_SPHERE) {
        // voxelShapes.c:288-335
        const float fx = px - p.center[0], fy = py - p.center[1], fz = pz - p.center[2];
        const float d2 = fx * fx + fy * fy + fz * fz;
        uint32_t cls = 0;
        if (d2 < p.r2) cls = 1;
        else if (p.removing && p.flipNormals && d2 < p.r12) cls = 2;
        if (cls == 0 || (cls == 1 && p.removing)) return cls;
        const float mx = fmaxf(fmaxf(fabsf(fx), fabsf(fy)), fabsf(fz));
        const float k = 1.0f / mx;
        n[0] = fx * k; n[1] = fy * k; n[2] = fz * k;
        return cls;
    }
    // voxelShapes.c:191-225 with the normal of 131-147
    const V3 t = xform(p.invTransform, px, py, pz, 1.0f);
    const float dist = shape_sdf(p, t);
    uint32_t cls = 0;
    if (dist < 0.0f) cls = 1;
    else if (dist < 1.0f && p.removing && p.flipNormals) cls = 2;
    if (cls == 0 || (cls == 1 && p.removing)) return cls;
    const float h = 0.01f;
    const float x = shape_sdf(p, xform(p.invTransform, px + h, py + 0.0f, pz + 0.0f, 1.0f + 0.0f)) - dist;
    const float y = shape_sdf(p, xform(p.invTransform, px + 0.0f, py + h, pz + 0.0f, 1.0f + 0.0f)) - dist;
    const float z = shape_sdf(p, xform(p.invTransform, px + 0.0f, py + 0.0f, pz + h, 1.0f + 0.0f)) - dist;
    const float mx = fmaxf(fmaxf(fabsf(x), fabsf(y)), fabsf(z));
    const float k = 1.0f / mx;
    n[0] = x * k; n[1] = y * k; n[2] = z * k;
    return cls;
}

struct ShapeArgs {
    dn_shape_params p;
    uint32_t nx, ny;            // chunks of the range along x and y
    uint32_t* counts;           // per chunk (pass 1)
    const uint64_t* offsets;    // per chunk, exclusive prefix of counts (pass 2)
    dn_shape_hit* hits;
    uint64_t capacity;
};

// chunk of this block and the voxel of this thread (thread t <-> local index x + 8*(y + 8*z))
__device__ __forceinline__ uint32_t block_voxel(const ShapeArgs& a, int& gx, int& gy, int& gz)
{
    const uint32_t c = blockIdx.x;
    const uint32_t cx = c % a.nx, cy = (c / a.nx) % a.ny, cz = c / (a.nx * a.ny);
    const uint32_t t = threadIdx.x;
    gx = (a.p.chunkMin[0] + (int)cx) * 8 + (int)(t & 7u);
    gy = (a.p.chunkMin[1] + (int)cy) * 8 + (int)((t >> 3) & 7u);
    gz = (a.p.chunkMin[2] + (int)cz) * 8 + (int)(t >> 6);
    return c;
}

__global__ void __launch_bounds__(512) k_shape_count(ShapeArgs a)
{
    int gx, gy, gz;
    const uint32_t c = block_voxel(a, gx, gy, gz);
    float n[3];
    const uint32_t cls = shape_classify(a.p, gx, gy, gz, n);
    const int total = __syncthreads_count(cls != 0u);
    if (threadIdx.x == 0) a.counts[c] = (uint32_t)total;
}

__global__ void __launch_bounds__(512) k_shape_write(ShapeArgs a)
{
    __shared__ uint32_t warpCount[16];
    int gx, gy, gz;
    const uint32_t c = block_voxel(a, gx, gy, gz);
    float n[3];
    const uint32_t cls = shape_classify(a.p, gx, gy, gz, n);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned ballot = __ballot_sync(0xFFFFFFFFu, cls != 0u);
    if (lane == 0) warpCount[warp] = (uint32_t)__popc(ballot);
    __syncthreads();
    if (cls == 0u) return;
    uint32_t rank = (uint32_t)__popc(ballot & ((1u << lane) - 1u));
    for (uint32_t w = 0; w < warp; w++) rank += warpCount[w];
    const uint64_t at = a.offsets[c] + rank;
    if (at >= a.capacity) return;     // the host sized the list from pass 1; never taken
    dn_shape_hit h;
    h.local = (uint16_t)threadIdx.x;
    h.inside = cls == 1u ? 1u : 0u;
    h.pad = 0;
    h.normal[0] = n[0]; h.normal[1] = n[1]; h.normal[2] = n[2];
    a.hits[at] = h;
}

// device time of the evaluation passes and voxels evaluated, since the last reset
double g_shapeMs = 0.0;
unsigned long long g_shapeVoxels = 0;

}  // namespace

extern "C" void dn_cuda_shape_stats(uint64_t* voxels, double* deviceMs, int reset)
{
    if (voxels) *voxels = g_shapeVoxels;
    if (deviceMs) *deviceMs = g_shapeMs;
    if (reset) { g_shapeVoxels = 0; g_shapeMs = 0.0; }
}

namespace {

// Per-thread buffers of the evaluation, grown as needed and kept between calls (a shape call then costs
// two launches and three copies, no allocation): device counts / offsets / hits, pinned host offsets and
// hits, a stream and four timing events.  A shape call made from inside a transform function while the
// thread's buffers are still lent out (between dn_cuda_shape_eval and dn_cuda_shape_free) uses buffers
// of its own for that call.  The buffers are not freed at thread exit.
struct ShapeScratch {
    bool busy;
    int device;
    cudaStream_t stream;
    cudaEvent_t ev[4];
    uint32_t* dcounts; size_t nCounts;
    uint64_t* doffsets; size_t nOffsets;
    dn_shape_hit* dhits; size_t nHits;
    uint64_t* hoffsets; size_t nHOffsets;
    dn_shape_hit* hhits; size_t nHHits;
};
thread_local ShapeScratch t_scratch = {};

template <class T> int grow_device(T*& p, size_t& cap, size_t need)
{
    if (need <= cap && p) return DN_CUDA_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t n = need < 1024 ? 1024 : need + need / 2;
    COUNT_ALLOC();
    CK(cudaMalloc((void**)&p, n * sizeof(T)));
    cap = n;
    return DN_CUDA_OK;
}

template <class T> int grow_pinned(T*& p, size_t& cap, size_t need)
{
    if (need <= cap && p) return DN_CUDA_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const size_t n = need < 1024 ? 1024 : need + need / 2;
    COUNT_ALLOC();
    CK(cudaMallocHost((void**)&p, n * sizeof(T)));
    cap = n;
    return DN_CUDA_OK;
}

int scratch_ready(ShapeScratch& sc)
{
    if (sc.device == g_device && sc.stream) return DN_CUDA_OK;
    sc = ShapeScratch{};     // buffers of another device are left to it
    CK(cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking));
    for (auto& e : sc.ev) CK(cudaEventCreate(&e));
    sc.device = g_device;
    return DN_CUDA_OK;
}

// the two passes on sc; hits land in sc.hhits (pinned)
int shape_eval_on(ShapeScratch& sc, const ShapeArgs& proto, int64_t nchunks, uint32_t* counts, uint64_t* total)
{
    ShapeArgs a = proto;
    int rc = grow_device(sc.dcounts, sc.nCounts, (size_t)nchunks);
    if (!rc) rc = grow_device(sc.doffsets, sc.nOffsets, (size_t)nchunks);
    if (!rc) rc = grow_pinned(sc.hoffsets, sc.nHOffsets, (size_t)nchunks);
    if (rc) return rc;
    a.counts = sc.dcounts;
    COUNT_LAUNCH();
    CK(cudaEventRecord(sc.ev[0], sc.stream));
    k_shape_count<<<(unsigned)nchunks, 512, 0, sc.stream>>>(a);
    CK(cudaGetLastError());
    CK(cudaEventRecord(sc.ev[1], sc.stream));
    CK(cudaMemcpyAsync(counts, sc.dcounts, (size_t)nchunks * 4, cudaMemcpyDeviceToHost, sc.stream));
    CK(cudaStreamSynchronize(sc.stream));
    float msCount = 0.0f, msWrite = 0.0f;
    cudaEventElapsedTime(&msCount, sc.ev[0], sc.ev[1]);
    uint64_t sum = 0;
    for (int64_t i = 0; i < nchunks; i++) { sc.hoffsets[i] = sum; sum += counts[i]; }
    if (sum) {
        rc = grow_device(sc.dhits, sc.nHits, (size_t)sum);
        if (!rc) rc = grow_pinned(sc.hhits, sc.nHHits, (size_t)sum);
        if (rc) return rc;
        CK(cudaMemcpyAsync(sc.doffsets, sc.hoffsets, (size_t)nchunks * 8, cudaMemcpyHostToDevice, sc.stream));
        a.offsets = sc.doffsets;
        a.hits = sc.dhits;
        a.capacity = sum;
        COUNT_LAUNCH();
        CK(cudaEventRecord(sc.ev[2], sc.stream));
        k_shape_write<<<(unsigned)nchunks, 512, 0, sc.stream>>>(a);
        CK(cudaGetLastError());
        CK(cudaEventRecord(sc.ev[3], sc.stream));
        CK(cudaMemcpyAsync(sc.hhits, sc.dhits, (size_t)sum * sizeof(dn_shape_hit), cudaMemcpyDeviceToHost, sc.stream));
        CK(cudaStreamSynchronize(sc.stream));
        cudaEventElapsedTime(&msWrite, sc.ev[2], sc.ev[3]);
    } else if (!sc.hhits) {
        rc = grow_pinned(sc.hhits, sc.nHHits, 1);
        if (rc) return rc;
    }
    g_shapeMs += (double)msCount + (double)msWrite;
    g_shapeVoxels += (unsigned long long)nchunks * 512ull;
    *total = sum;
    return DN_CUDA_OK;
}

void scratch_release(ShapeScratch& sc)
{
    for (auto& e : sc.ev) if (e) cudaEventDestroy(e);
    if (sc.stream) cudaStreamDestroy(sc.stream);
    cudaFree(sc.dcounts); cudaFree(sc.doffsets); cudaFree(sc.dhits);
    cudaFreeHost(sc.hoffsets);
    sc = ShapeScratch{};
}

}  // namespace

extern "C" int dn_cuda_shape_eval(const dn_shape_params* p, uint32_t* counts, dn_shape_hit** hits, uint64_t* total)
{
    if (!p || !counts || !hits || !total) return dn_set_err(DN_CUDA_ERR_ARG, "null argument");
    *hits = nullptr;
    *total = 0;
    if (p->kind > DN_SHAPE_PYRAMID) return dn_set_err(DN_CUDA_ERR_ARG, "unknown shape kind %u", p->kind);
    int64_t n[3];
    for (int i = 0; i < 3; i++) {
        if (p->chunkMin[i] < 0 || p->chunkMax[i] < p->chunkMin[i])
            return dn_set_err(DN_CUDA_ERR_ARG, "bad chunk range");
        n[i] = (int64_t)p->chunkMax[i] - p->chunkMin[i] + 1;
    }
    const int64_t nchunks = n[0] * n[1] * n[2];
    if (nchunks > 0x7FFFFFFF) return dn_set_err(DN_CUDA_ERR_ARG, "chunk range too large");
    CK(cudaSetDevice(g_device));
    ShapeArgs a;
    memset(&a, 0, sizeof(a));
    a.p = *p;
    a.nx = (uint32_t)n[0];
    a.ny = (uint32_t)n[1];
    ShapeScratch& sc = t_scratch;
    if (!sc.busy) {
        int rc = scratch_ready(sc);
        if (!rc) rc = shape_eval_on(sc, a, nchunks, counts, total);
        if (rc) return rc;
        sc.busy = true;
        *hits = sc.hhits;
        return DN_CUDA_OK;
    }
    // nested call (from a transform function): buffers of its own, the hits copied to malloc'd memory
    ShapeScratch tmp = {};
    int rc = scratch_ready(tmp);
    if (!rc) rc = shape_eval_on(tmp, a, nchunks, counts, total);
    dn_shape_hit* out = nullptr;
    if (!rc) {
        out = (dn_shape_hit*)malloc((size_t)(*total ? *total : 1) * sizeof(dn_shape_hit));
        if (!out) rc = dn_set_err(DN_CUDA_ERR_NOMEM, "no host memory for %llu shape hits", (unsigned long long)*total);
        else memcpy(out, tmp.hhits, (size_t)*total * sizeof(dn_shape_hit));
    }
    cudaFreeHost(tmp.hhits);
    scratch_release(tmp);
    if (rc) return rc;
    *hits = out;
    return DN_CUDA_OK;
}

extern "C" void dn_cuda_shape_free(dn_shape_hit* hits)
{
    ShapeScratch& sc = t_scratch;
    if (sc.busy && hits == sc.hhits) sc.busy = false;
    else free(hits);
}
