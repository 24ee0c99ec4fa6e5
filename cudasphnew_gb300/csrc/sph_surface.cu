// Surface particles (CreateIsParticleSurfaceList, particle_simulation.cu:
// 1818-1839).  The reference allocates the flags and hands them to its force
// kernel, which never writes them; the kernel does sum the neighbours'
// positions and count them (:371-379, unused), and the parameters carry the
// "surface extraction threshold parameters" cmDistanceThresh and nPartTresh
// (particle_simulation.h:102-104).  Here a particle is a surface particle
// when it has fewer than nPartTresh neighbours within h, or when the centre
// of mass of those neighbours lies farther than cmDistanceThresh * h from it.
// Computed from the sorted pre-step state of the last step.
#include "sph_device.cuh"
#include "sph_sim.h"

namespace sph {
namespace {

__global__ void k_surface(int n, const float4* __restrict__ posS, const int* __restrict__ workIds, RowTables T,
                          GridDev g_, float h_, float cmThresh, float countThresh, int* __restrict__ flags) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    const float4 xi = posS[u];
    const SceneDev* S = T.scenes ? T.scenes + __float_as_int(xi.w) : nullptr;
    const GridDev& g = S ? S->g : g_;
    const float h = S ? S->ph.h : h_;
    const float h2 = h * h;
    const Stencil st = stencil(xi, h, g);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int cnt = 0;
    for (int r = 0; r < 9; r++) {
        int s, e;
        row_range(xi, st, h, g, T, true, r, s, e);
        for (int t = s; t < e; t++) {
            const float4 xj = posS[t];
            const float r2 = dist2(xi, xj);
            if (t == u || !(r2 <= h2)) continue;
            sx += xj.x;
            sy += xj.y;
            sz += xj.z;
            cnt++;
        }
    }
    bool surface = (float)cnt < countThresh;
    if (cnt > 0) {
        const double cx = sx / cnt - xi.x, cy = sy / cnt - xi.y, cz = sz / cnt - xi.z;
        surface = surface || sqrt(cx * cx + cy * cy + cz * cz) > (double)cmThresh * h;
    }
    flags[workIds[u]] = surface ? 1 : 0;
}

// The same test over the reused neighbour lists (after a step that ran over
// them the sorted copies are in the lists' working order, which the cell
// tables do not describe): the candidates within the skin radius are a
// superset of those within h, visited in the lists' order.
__global__ void k_surface_lists(int n, const float4* __restrict__ posS, const int* __restrict__ workIds,
                                NeighbourLists L, float h, float cmThresh, float countThresh, int* __restrict__ flags) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    const float4 xi = posS[u];
    const float h2 = h * h;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int cnt = 0;
    const int rows = L.rows[u];
    for (int r = 0; r < rows; r++) {
        const size_t at = (size_t)r * n + u;
        const int sv = L.start[at];
        const uint2 m2 = L.skin[at];
        const unsigned long long m = (unsigned long long)m2.x | ((unsigned long long)m2.y << 32);
        const int t0 = sv & 0x7fffffff;
        const int t1 = sv < 0 ? (int)m2.x : t0 + 64;
        for (int t = t0; t < t1; t++) {
            if (sv >= 0 && !((m >> (t - t0)) & 1ull)) continue;
            const float4 xj = posS[t];
            const float r2 = dist2(xi, xj);
            if (t == u || !(r2 <= h2)) continue;
            sx += xj.x;
            sy += xj.y;
            sz += xj.z;
            cnt++;
        }
    }
    bool surface = (float)cnt < countThresh;
    if (cnt > 0) {
        const double cx = sx / cnt - xi.x, cy = sy / cnt - xi.y, cz = sz / cnt - xi.z;
        surface = surface || sqrt(cx * cx + cy * cy + cz * cz) > (double)cmThresh * h;
    }
    flags[workIds[u]] = surface ? 1 : 0;
}

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" sph_status sph_surface_particles(sph_handle s, int* flags) {
    if (!s || !flags) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->stepped) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no step has run yet");
    if (s->numScenes > 1) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "surface flags are per scene: not for batched handles");
    int* d = nullptr;
    SPH_CUDA(dalloc(&d, (size_t)s->n));
    GridDev g = grid_of(s);
    const float4* posS = s->posS;
    float4* absS = nullptr;
    if (g.rel) {  // cell-relative positions: search an absolute copy
        cudaError_t ea = dalloc(&absS, (size_t)s->n);
        if (ea != cudaSuccess) {
            cudaFree(d);
            SPH_CUDA(ea);
        }
        launch_rel_to_abs(s->n, s->posS, g, nullptr, 0, absS, s->stream);
        posS = absS;
        g.rel = 0;
    }
    if (s->vlOn && s->lastStepLists)
        k_surface_lists<<<(s->n + 127) / 128, 128, 0, s->stream>>>(s->n, posS, s->sb.workIds, s->vl,
                                                                   s->P.compactSupport, s->P.cmDistanceThresh,
                                                                   s->P.nPartTresh, d);
    else
        k_surface<<<(s->n + 127) / 128, 128, 0, s->stream>>>(s->n, posS, s->sb.workIds, rows_of(s), g,
                                                             s->P.compactSupport, s->P.cmDistanceThresh,
                                                             s->P.nPartTresh, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, d, sizeof(int) * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (absS) cudaFree(absS);
    SPH_CUDA(e);
    return latched_status(s);
}
