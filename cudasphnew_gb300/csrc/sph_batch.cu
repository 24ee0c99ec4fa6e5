// Batched scenes: one handle holding many independent simulations
// (sph_create_batch, sph_batch_info).  No reference counterpart.
//
// Layout.  The scenes' particles are concatenated, scene after scene, in the
// handle's state arrays; each particle carries its scene index in the .w lane
// of its position.  The scenes' cell grids are concatenated too: scene k's
// cells are numbered from its cellBase, so one counting sort and one cell
// scan serve all scenes and no cell holds particles of two scenes.  The
// step's kernels are the single-scene kernels in their batched form: each
// particle reads its scene's grid, constants and boundary maps from a device
// table.  With reused neighbour lists every scene keeps its own build
// decision (its own displacement and h).  A scene's arithmetic is exactly
// that of a handle holding only it, so its results are bit-identical to
// running it alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <new>
#include <vector>

#include "sph_sim.h"

using namespace sph;

extern "C" {

sph_status sph_create_batch(const sph_scene* scenes, int numScenes, const sph_options* opts, sph_handle* out) {
    if (!out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!scenes || numScenes < 1) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no scenes");
    sph_options O;
    if (opts) O = *opts;
    else sph_default_options(&O);
    if (O.cellRelative) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "batched handles keep absolute positions");
    long long n = 0, C = 0;
    size_t mapNodes = 0;
    float tension = 0.0f;
    std::vector<unsigned int> dims((size_t)3 * numScenes, 0u);
    for (int k = 0; k < numScenes; k++) {
        const sph_scene& sc = scenes[k];
        sph_status st = validate_params(sc.params, &O);
        if (st) return st;
        if (!sc.vertexData) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "a scene's vertexData is NULL");
        if (sc.boundary) {
            st = check_desc(sc.boundary, &dims[(size_t)3 * k]);
            if (st) return st;
            mapNodes += (size_t)dims[3 * k] * dims[3 * k + 1] * dims[3 * k + 2];
        }
        n += sc.params->numParticles;
        C += (long long)sc.params->gridDim[0] * sc.params->gridDim[1] * sc.params->gridDim[2];
        tension = std::max(tension, std::fabs(sc.params->tensionCoefficient));
    }
    if (n > (1ll << 30)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "more than 2^30 particles in the batch");
    if (C > (long long)INT_MAX - 2 * SCAN_TILE) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "too many cells in the batch");

    sph_sim* s = new (std::nothrow) sph_sim();
    if (!s) SPH_FAIL(SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    // the handle's own parameters: scene 0's, with the batch's particle count;
    // the tension coefficient only selects whether the force kernel computes
    // the colour field (every constant comes from the scene table)
    s->P = *scenes[0].params;
    s->P.numParticles = (unsigned int)n;
    s->P.tensionCoefficient = tension;
    s->O = O;
    s->numScenes = numScenes;
    std::vector<SceneDev> table((size_t)numScenes);
    auto bail = [&](sph_status st) {
        free_all(s);
        delete s;
        return st;
    };
#define BATCH_CUDA(call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return bail(record_error(e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA, \
                                     __FILE__, __LINE__, cudaGetErrorString(e_)));                    \
    } while (0)
    sph_status st = alloc_handle(s, (int)n, C);
    if (st) return bail(st);
    if (mapNodes) {
        BATCH_CUDA(dalloc(&s->map4, mapNodes));
        BATCH_CUDA(dalloc(&s->mapDist, mapNodes));
    }
    cudaStream_t q = s->stream;
    size_t pOff = 0, mOff = 0;
    long long cOff = 0;
    s->sceneStart.assign(1, 0u);
    s->sceneCell.assign(1, 0u);
    for (int k = 0; k < numScenes; k++) {
        const sph_scene& sc = scenes[k];
        const SimulationParameters& P = *sc.params;
        const int nk = (int)P.numParticles;
        SceneDev& d = table[(size_t)k];
        d.g = make_grid(P, false);
        d.g.cellBase = (int)cOff;
        d.ph = make_phys(P, O);
        d.map = MapDev{};
        if (sc.boundary) {
            const unsigned int* dk = &dims[(size_t)3 * k];
            BATCH_CUDA(launch_build_maps(*sc.boundary, dk, s->mapDist + mOff, nullptr, nullptr, s->map4 + mOff, q));
            d.map = map_of(*sc.boundary, dk, s->map4 + mOff, s->mapDist + mOff);
            mOff += (size_t)dk[0] * dk[1] * dk[2];
        }
        // initial state, stream-ordered through the staging buffer
        BATCH_CUDA(cudaMemcpyAsync(s->staging, sc.vertexData, sizeof(float) * 3 * (size_t)nk, cudaMemcpyHostToDevice,
                                   q));
        launch_unpack_aos(s->staging, 3, 0, nk, s->pos + pOff, q);
        launch_set_scene(s->pos + pOff, nk, k, q);
        if (sc.simulationData) {
            BATCH_CUDA(cudaMemcpyAsync(s->staging, sc.simulationData, sizeof(float) * 10 * (size_t)nk,
                                       cudaMemcpyHostToDevice, q));
            launch_unpack_aos(s->staging, 10, 6, nk, s->vel + pOff, q);
            for (int i = 0; i < nk; i++) {
                s->sdMass[pOff + i] = sc.simulationData[(size_t)i * 10 + 0];
                s->sdEnergy[pOff + i] = sc.simulationData[(size_t)i * 10 + 9];
            }
        }
        pOff += (size_t)nk;
        cOff += (long long)d.g.numCells;
        s->sceneStart.push_back((unsigned int)pOff);
        s->sceneCell.push_back((unsigned int)cOff);
    }
    BATCH_CUDA(dalloc(&s->scenesDev, (size_t)numScenes));
    BATCH_CUDA(cudaMemcpyAsync(s->scenesDev, table.data(), sizeof(SceneDev) * table.size(), cudaMemcpyHostToDevice,
                               q));
    s->sb.scenes = s->scenesDev;
    // reused neighbour lists, one build decision per scene
    if (sph_status sl = alloc_lists(s)) return bail(sl);
    BATCH_CUDA(cudaGetLastError());
    BATCH_CUDA(cudaStreamSynchronize(q));  // `table` leaves scope
#undef BATCH_CUDA
    *out = s;
    return SPH_OK;
}

sph_status sph_batch_info(sph_handle s, int* numScenes, unsigned int* firstParticle, unsigned int* firstCell) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (numScenes) *numScenes = s->numScenes;
    for (int k = 0; k <= s->numScenes; k++) {
        const bool single = s->sceneStart.empty();
        if (firstParticle) firstParticle[k] = single ? (k ? (unsigned int)s->n : 0u) : s->sceneStart[(size_t)k];
        if (firstCell) firstCell[k] = single ? (k ? (unsigned int)s->numCellsTotal : 0u) : s->sceneCell[(size_t)k];
    }
    return SPH_OK;
}

}  // extern "C"
