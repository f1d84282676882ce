// pin_harness.cpp -- TEST INFRASTRUCTURE.  Runs the reference's own compute shaders, translated to C++
// by glsl_to_cpp.py, invocation by invocation on the CPU, so that the CPU oracle can be pinned to them.
//
// pin_draw:  one voxelDraw.comp invocation per pixel of the reference's w/16 x h/16 dispatch
//            (voxel.c:879); returns the stored RGBA (gamma-corrected colour, depth) and the tile flags.
// pin_light: one voxelLighting.comp invocation per (request word, local id) (voxel.c:950); returns the
//            FP32 specular and diffuse light each invocation computed, captured after the shader clamps
//            them and before it quantises them into the voxel words.  Every invocation runs against the
//            buffers as they were before the dispatch (they are restored after each one): that is the
//            oracle's deterministic reading of the dispatch (committed-lighting reads, per-launch sample
//            count), where the reference's own GPU run reads and writes them in place in an undefined order.
#include "glsl_shim.hpp"
#include <vector>

static float g_capSpec[3], g_capDiff[3];
static glsl::uint g_capIndex = 0xFFFFFFFFu;
static bool g_captured = false;

namespace shader_light {
using glsl::uint;
struct uvec3c { uint x, y, z; };
static glsl::uvec3 gl_WorkGroupID, gl_LocalInvocationID, gl_WorkGroupSize(32u, 1u, 1u);
inline void pin_capture(uint index, const glsl::vec3& spec, const glsl::vec3& diff)
{
    g_capIndex = index;
    g_capSpec[0] = spec.x; g_capSpec[1] = spec.y; g_capSpec[2] = spec.z;
    g_capDiff[0] = diff.x; g_capDiff[1] = diff.y; g_capDiff[2] = diff.z;
    g_captured = true;
}
#include "shader_light.inc"
}

namespace shader_draw {
using glsl::uint;
static glsl::uvec3 gl_GlobalInvocationID;
#include "shader_draw.inc"
}

extern "C" {

struct PinMap {
    uint32_t sx, sy, sz;
    const uint32_t* handles;     // 3 words per tile: flags, lastUsed, voxelIndex
    const uint32_t* chunks;      // 23 words per tile: pos[3], numIndirectSamples, partialCounts[3], bitMask[16]
    const uint32_t* voxels;      // 4 words per voxel: normal, albedo, specLight, diffuseLight
    uint32_t nvox;
    const uint32_t* materials;   // 256 x 8 words (voxel.h:82-94 layout)
    float skyBot[3], skyTop[3], sunStrength[3], ambient[3];
};

}

template <class NS_Chunk, class NS_Handle, class NS_Voxel, class NS_Material>
static void load_buffers(const PinMap* pm, std::vector<NS_Handle>& h, std::vector<NS_Chunk>& c, std::vector<NS_Voxel>& v,
                         std::vector<NS_Material>& mats)
{
    const size_t tiles = (size_t)pm->sx * pm->sy * pm->sz;
    h.resize(tiles); c.resize(tiles); v.resize(pm->nvox ? pm->nvox : 1); mats.resize(256);
    for (size_t t = 0; t < tiles; t++) {
        h[t].flags = pm->handles[3 * t]; h[t].lastUsed = pm->handles[3 * t + 1]; h[t].voxelIndex = pm->handles[3 * t + 2];
        const uint32_t* w = &pm->chunks[23 * t];
        c[t].pos = glsl::ivec3((int)w[0], (int)w[1], (int)w[2]);
        c[t].numIndirectSamples = w[3];
        for (int k = 0; k < 3; k++) c[t].partialCounts[k] = w[4 + k];
        for (int k = 0; k < 16; k++) c[t].bitMask[k] = w[7 + k];
    }
    for (uint32_t i = 0; i < pm->nvox; i++) {
        v[i].normal = pm->voxels[4 * i]; v[i].albedo = pm->voxels[4 * i + 1];
        v[i].specLight = pm->voxels[4 * i + 2]; v[i].diffuseLight = pm->voxels[4 * i + 3];
    }
    for (int m = 0; m < 256; m++) {
        const uint32_t* w = &pm->materials[8 * m];
        float f[8];
        memcpy(f, w, sizeof(f));
        mats[m].padding = glsl::vec2(f[0], f[1]);
        mats[m].emissive = w[2] != 0;
        mats[m].opacity = f[3];
        mats[m].refractIndex = f[4];
        mats[m].specular = f[5];
        mats[m].reflectType = w[6];
        mats[m].shininess = w[7];
    }
}

extern "C" void pin_draw(const PinMap* pm, const float invView[16], const float invCV[16], const float invProj[16],
                         uint32_t w, uint32_t hgt, uint32_t viewMode, float* outRGBA, uint32_t* outFlags)
{
    using namespace shader_draw;
    std::vector<ChunkHandle> h; std::vector<Chunk> c; std::vector<CompressedVoxel> v; std::vector<Material> mats;
    load_buffers(pm, h, c, v, mats);
    map.p = h.data(); map.n = h.size();
    chunks.p = c.data(); chunks.n = c.size();
    voxels.p = v.data(); voxels.n = pm->nvox;
    materials.p = mats.data(); materials.n = 256;
    std::vector<glsl::vec4> px((size_t)w * hgt, glsl::vec4(0.0f, 0.0f, 0.0f, -1.0f));
    colorOutput.px = px.data(); colorOutput.w = (int)w; colorOutput.h = (int)hgt;
    mapSize = glsl::uvec3(pm->sx, pm->sy, pm->sz);
    useCubemap = false;
    skyGradientBot = glsl::vec3(pm->skyBot[0], pm->skyBot[1], pm->skyBot[2]);
    skyGradientTop = glsl::vec3(pm->skyTop[0], pm->skyTop[1], pm->skyTop[2]);
    sunStrength = glsl::vec3(pm->sunStrength[0], pm->sunStrength[1], pm->sunStrength[2]);
    ambientStrength = glsl::vec3(pm->ambient[0], pm->ambient[1], pm->ambient[2]);
    memcpy(invViewMat.m, invView, 64);
    memcpy(invCenteredViewMat.m, invCV, 64);
    memcpy(invProjectionMat.m, invProj, 64);
    composeRasterized = false;
    shader_draw::viewMode = viewMode;
    const uint32_t gx = w / 16u, gy = hgt / 16u;     // the reference dispatches w/16 x h/16 groups of 16x16
    for (uint32_t y = 0; y < gy * 16u; y++)
        for (uint32_t x = 0; x < gx * 16u; x++) {
            reset_globals();
            gl_GlobalInvocationID = glsl::uvec3(x, y, 0u);
            shader_main();
        }
    for (size_t i = 0; i < px.size(); i++) {
        outRGBA[4 * i] = px[i].x; outRGBA[4 * i + 1] = px[i].y; outRGBA[4 * i + 2] = px[i].z; outRGBA[4 * i + 3] = px[i].w;
    }
    for (size_t t = 0; t < h.size(); t++) outFlags[t] = h[t].flags;
}

extern "C" void pin_light(const PinMap* pm, const uint32_t* requests, uint32_t nreq, float t, uint32_t numDiffuse,
                          uint32_t maxDiffuse, uint32_t diffuseLimit, uint32_t specLimit, const float sunDirN[3],
                          float softness, const float cam[3], float* outSpec, float* outDiff, uint8_t* outValid)
{
    using namespace shader_light;
    std::vector<ChunkHandle> h; std::vector<Chunk> c; std::vector<CompressedVoxel> v; std::vector<Material> mats;
    load_buffers(pm, h, c, v, mats);
    const std::vector<ChunkHandle> h0 = h;
    const std::vector<Chunk> c0 = c;
    const std::vector<CompressedVoxel> v0 = v;
    std::vector<uint> req(requests, requests + nreq);
    map.p = h.data(); map.n = h.size();
    chunks.p = c.data(); chunks.n = c.size();
    voxels.p = v.data(); voxels.n = pm->nvox;
    materials.p = mats.data(); materials.n = 256;
    chunkIndices.p = req.data(); chunkIndices.n = req.size();
    mapSize = glsl::uvec3(pm->sx, pm->sy, pm->sz);
    useCubemap = false;
    skyGradientBot = glsl::vec3(pm->skyBot[0], pm->skyBot[1], pm->skyBot[2]);
    skyGradientTop = glsl::vec3(pm->skyTop[0], pm->skyTop[1], pm->skyTop[2]);
    sunStrength = glsl::vec3(pm->sunStrength[0], pm->sunStrength[1], pm->sunStrength[2]);
    ambientStrength = glsl::vec3(pm->ambient[0], pm->ambient[1], pm->ambient[2]);
    time = t;
    numDiffuseSamples = numDiffuse;
    maxDiffuseSamples = maxDiffuse;
    diffuseBounceLimit = diffuseLimit;
    specularBounceLimit = specLimit;
    sunDir = glsl::vec3(sunDirN[0], sunDirN[1], sunDirN[2]);
    shadowSoftness = softness;
    camPos = glsl::vec3(cam[0], cam[1], cam[2]);
    for (uint32_t i = 0; i < pm->nvox; i++) outValid[i] = 0;
    for (uint32_t r = 0; r < nreq; r++)
        for (uint32_t l = 0; l < 32u; l++) {
            reset_globals();
            gl_WorkGroupID = glsl::uvec3(r, 0u, 0u);
            gl_LocalInvocationID = glsl::uvec3(l, 0u, 0u);
            g_captured = false;
            shader_main();
            if (g_captured && g_capIndex < pm->nvox) {
                memcpy(&outSpec[3 * g_capIndex], g_capSpec, 12);
                memcpy(&outDiff[3 * g_capIndex], g_capDiff, 12);
                outValid[g_capIndex] = 1;
            }
            std::copy(h0.begin(), h0.end(), h.begin());
            std::copy(c0.begin(), c0.end(), c.begin());
            std::copy(v0.begin(), v0.end(), v.begin());
        }
}
