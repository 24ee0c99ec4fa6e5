// C ABI of the GB300 SPH step: handle management, the per-step stage
// sequence, read-back and boundary-map set-up.  See include/sph.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "sph_sim.h"

using namespace sph;

namespace {

thread_local std::string g_lastError;

// The reference's error message shape (util.h:24-39).
sph_status fail(sph_status st, const char* file, int line, const std::string& msg) {
    std::ostringstream s;
    s << "Exception thrown in FILE: " << file << " LINE: " << line << "\n"
      << "Error Message: " << msg << "\n";
    g_lastError = s.str();
    return st;
}

const char* kStageNames[ST_COUNT] = {"hash_count", "cell_scan",   "scatter",     "rank_gather",
                                     "density",    "force_integrate", "ts_children", "sub_sort",
                                     "sub_density", "sub_force"};

}  // namespace

namespace sph {
// Records a failure in the per-thread message sph_last_error() returns, for
// entry points defined in other translation units.
sph_status record_error(sph_status st, const char* file, int line, const std::string& msg) {
    return fail(st, file, line, msg);
}
}  // namespace sph


namespace sph {

// The device address of page-locked host memory (pinned or registered),
// which kernels read and write directly over the host link; NULL for
// pageable memory, which goes through the staging buffer.
void* host_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory on older drivers: clear the error
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

RowTables rows_of(const sph_sim* s) {
    return RowTables{s->sb.cellOffset, s->sb.halfOffset, s->sb.scenes, s->sb.skip};
}

GridDev make_grid(const SimulationParameters& P, bool sub) {
    GridDev g;
    for (int a = 0; a < 3; a++) {
        g.origin[a] = P.gridOrigin[a];
        g.dim[a] = sub ? P.gridDimSubParticles[a] : P.gridDim[a];
    }
    g.spacing = sub ? P.gridSpacingSubParticles : P.gridSpacing;
    g.numCells = g.dim[0] * g.dim[1] * g.dim[2];
    g.cellBase = 0;
    g.rel = 0;
    return g;
}

PhysDev make_phys(const SimulationParameters& P, const sph_options& O) {
    PhysDev ph;
    ph.h = P.compactSupport;
    ph.h2 = P.compactSupport * P.compactSupport;
    ph.poly6m = P.poly6 * P.particleMass;
    ph.mass = P.particleMass;
    ph.stiffness = P.gasStiffness;
    ph.restDensity = P.restDensity;
    ph.pressCoef = -P.particleMass * P.gradSpiky;
    ph.viscCoef = P.dynamicViscosity * P.particleMass * P.laplVisc;
    ph.cgCoef = P.particleMass * P.gradPoly6;
    ph.clCoef = P.particleMass * P.laplPoly6;
    ph.tension = P.tensionCoefficient;
    ph.normThresh = P.normThresh;
    ph.dt = P.timeStep;
    ph.dtCollide = P.timeStep;
    ph.gravity = P.gravity;
    ph.gravityAxis = O.gravityAxis;
    for (int a = 0; a < 3; a++) {
        ph.boxCen[a] = P.boxCen[a];
        ph.boxDim[a] = P.boxDim[a];
    }
    ph.restitution = P.restitution;
    return ph;
}

sph_status validate_params(const SimulationParameters* P, const sph_options* O) {
    if (!P) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "params is NULL");
    if (P->numParticles == 0 || P->numParticles > (1u << 30))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "numParticles must be in [1, 2^30]");
    double cells = 1.0;
    for (int a = 0; a < 3; a++) {
        if (P->gridDim[a] <= 0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "gridDim must be positive");
        cells *= P->gridDim[a];
    }
    if (cells > 2147483000.0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "too many grid cells");
    if (!(P->gridSpacing > 0.0f) || !(P->compactSupport > 0.0f))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "gridSpacing and compactSupport must be positive");
    if (P->compactSupport > P->gridSpacing)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT,
                 "compactSupport exceeds gridSpacing: the 27-cell stencil would miss neighbours");
    if (O && (O->gravityAxis < 0 || O->gravityAxis > 2))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "gravityAxis must be 0, 1 or 2");
    if (O && (O->childMode < 0 || O->childMode > 1)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "childMode must be 0 or 1");
    if (O && (O->cellRelative < 0 || O->cellRelative > 1))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "cellRelative must be 0 or 1");
    // at most 0.4: the skin sphere then spans at most 4 cells per axis (compactSupport <= gridSpacing),
    // so a particle's rows fit the lists' VL_SLOTS = 16 entries
    if (O && !(O->neighbourSkin >= 0.0f && O->neighbourSkin <= 0.4f))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "neighbourSkin must be in [0, 0.4]");
    if (O && O->cellRelative &&
        (P->gridDim[0] > REL_MAX_X || P->gridDim[1] > REL_MAX_Y || P->gridDim[2] > REL_MAX_Z))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "cellRelative needs gridDim of at most 2048 x 2048 x 1024");
    return SPH_OK;
}

sph_status check_desc(const sph_boundary_desc* d, unsigned int dims[3]) {
    if (!d) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "boundary desc is NULL");
    if (d->numShapes < 1 || d->numShapes > 8)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "numShapes must be in [1, 8]");
    for (int i = 0; i < d->numShapes; i++) {
        int k = d->shapes[i].kind;
        if (k != SPH_SHAPE_SPHERE && k != SPH_SHAPE_CONE && k != SPH_SHAPE_BOX && k != SPH_SHAPE_MESH)
            SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown shape kind");
        if (k == SPH_SHAPE_MESH) {
            const float g = d->shapes[i].p[0];
            if (!d->sdfGrids || !(g >= 0.0f) || g >= (float)d->numSdfGrids || g != (float)(int)g)
                SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "a mesh shape names no grid of sdfGrids");
            const sph_sdf_grid& G = d->sdfGrids[(int)g];
            if (!G.distance || G.dims[0] == 0 || G.dims[1] == 0 || G.dims[2] == 0 || !(G.dx > 0.0f))
                SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "empty signed distance grid");
        }
    }
    if (!(d->gridSpacing > 0.0f) || !(d->particleSpacing > 0.0f) || !(d->compactSupport > 0.0f))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "boundary spacings must be positive");
    double total = 1.0;
    for (int a = 0; a < 3; a++) {
        if (!(d->gridEnd[a] > d->gridStart[a]))
            SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "invalid domain definition");  // SphInComplexShapes.cpp:43-47
        // SphInComplexShapes.cpp:49-54
        dims[a] = (unsigned int)((d->gridEnd[a] - d->gridStart[a]) / d->gridSpacing) + 1;
        total *= dims[a];
    }
    if (total > 512.0 * 1024 * 1024) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "boundary grid too large");
    return SPH_OK;
}

void free_all(sph_sim* s) {
    corrector_free(s);
    if (s->graphExec) cudaGraphExecDestroy(s->graphExec);
    if (s->graph) cudaGraphDestroy(s->graph);
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    void* ptrs[] = {s->pos, s->vel, s->posS, s->velS, s->rho4S, s->accS, s->sb.cnt, s->sb.cellOffset,
                    s->sb.keySlot, s->sb.tmpIds, s->sb.sortedHash, s->sb.sortedIds, s->sb.workIds,
                    s->sb.halfOffset, s->scanBlock,
                    s->status, s->staging, s->map4, s->mapDist, s->rowStart, s->rowMask, s->diagBuf,
                    s->scenesDev, s->reuse, s->vl.start, s->vl.skin, s->vl.exact, s->vl.rows, s->vl.posB,
                    s->vl.flags, s->vl.slotScene};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    void* tsPtrs[] = {s->ts.state,     s->ts.blockCounts, s->ts.counts,
                      s->ts.splitIds,  s->ts.boundaryIds, s->ts.defaultIds,  s->ts.subIds,
                      s->ts.subPos,    s->ts.subVel,      s->ts.subAcc,      s->ts.subRho,
                      s->ts.subCnt,    s->ts.subOffset,   s->ts.subKeySlot,  s->ts.subTmp,
                      s->ts.subSortedHash, s->ts.subSortedIds, s->ts.subPosS, s->ts.subVelS, s->ts.markList,
                      s->subScanBlock};
    for (void* p : tsPtrs)
        if (p) cudaFree(p);
    if (s->statusHost) cudaFreeHost(s->statusHost);
    for (cudaStream_t q : {s->upStream, s->downStream})
        if (q) {
            cudaStreamSynchronize(q);
            cudaStreamDestroy(q);
        }
    for (int k = 0; k < 2; k++) {
        if (s->upLand[k]) cudaFree(s->upLand[k]);
        if (s->upReady[k]) cudaEventDestroy(s->upReady[k]);
        if (s->upFree[k]) cudaEventDestroy(s->upFree[k]);
    }
    if (s->downStage) cudaFree(s->downStage);
    if (s->downReady) cudaEventDestroy(s->downReady);
    if (s->downFree) cudaEventDestroy(s->downFree);
    if (s->ownStream) cudaStreamDestroy(s->ownStream);
}

PhysDev make_sub_phys(const SimulationParameters& P, const sph_options& O) {
    PhysDev ph = make_phys(P, O);
    ph.h = P.compactSupportSub;
    ph.h2 = P.compactSupportSub * P.compactSupportSub;
    ph.poly6m = P.poly6Sub * P.subParticleMass;
    ph.mass = P.subParticleMass;
    ph.pressCoef = -P.subParticleMass * P.gradSpikySub;
    ph.viscCoef = P.dynamicViscosity * P.subParticleMass * P.laplViscSub;
    ph.cgCoef = P.subParticleMass * P.gradPoly6Sub;
    ph.clCoef = P.subParticleMass * P.laplPoly6Sub;
    ph.dt = P.timeStepSubParticles;
    ph.dtCollide = P.timeStep;  // collision_handling_sub_particles uses the coarse step (:916)
    return ph;
}

// Allocates the two-scale state on first use: 8n child slots and the fine
// level's counting-sort buffers.
sph_status ensure_two_scale(sph_sim* s) {
    if (s->tsReady) return SPH_OK;
    const size_t n = (size_t)s->n;
    const size_t n4 = (n + 3) & ~(size_t)3;
    const size_t nb = (n + 1023) / 1024;
    const size_t Cs = (size_t)s->P.gridDimSubParticles[0] * s->P.gridDimSubParticles[1] * s->P.gridDimSubParticles[2];
    const size_t tiles = (Cs + 1 + SCAN_TILE - 1) / SCAN_TILE;
    TwoScaleDev& T = s->ts;
    SPH_CUDA(dalloc(&T.state, n4));
    SPH_CUDA(dalloc(&T.blockCounts, 3 * nb));
    SPH_CUDA(dalloc(&T.counts, 5));
    SPH_CUDA(dalloc(&T.markList, n));
    SPH_CUDA(dalloc(&T.splitIds, n));
    SPH_CUDA(dalloc(&T.boundaryIds, n));
    SPH_CUDA(dalloc(&T.defaultIds, n));
    SPH_CUDA(dalloc(&T.subIds, 8 * n));
    SPH_CUDA(dalloc(&T.subPos, 8 * n));
    SPH_CUDA(dalloc(&T.subVel, 8 * n));
    SPH_CUDA(dalloc(&T.subAcc, 8 * n));
    SPH_CUDA(dalloc(&T.subRho, 8 * n));
    SPH_CUDA(dalloc(&T.subCnt, Cs + 1 + SCAN_TILE));
    SPH_CUDA(dalloc(&T.subOffset, Cs + 1 + SCAN_TILE));
    SPH_CUDA(dalloc(&T.subKeySlot, 8 * n));
    SPH_CUDA(dalloc(&T.subTmp, 8 * n));
    SPH_CUDA(dalloc(&T.subSortedHash, 8 * n));
    SPH_CUDA(dalloc(&T.subSortedIds, 8 * n));
    SPH_CUDA(dalloc(&T.subPosS, 8 * n));
    SPH_CUDA(dalloc(&T.subVelS, 8 * n));
    SPH_CUDA(dalloc(&s->subScanBlock, tiles + 2));
    cudaStream_t q = s->stream;
    // index buffers start valid (0): an entry a failed step leaves unwritten
    // still names a child slot or a fine cell
    for (int* p : {T.subTmp, T.subSortedHash, T.subSortedIds})
        SPH_CUDA(cudaMemsetAsync(p, 0, sizeof(int) * 8 * (size_t)n, q));
    SPH_CUDA(cudaMemsetAsync(T.state, 0, n4, q));
    SPH_CUDA(cudaMemsetAsync(T.counts, 0, sizeof(int) * 5, q));
    SPH_CUDA(cudaMemsetAsync(T.subPos, 0, sizeof(float4) * 8 * n, q));
    SPH_CUDA(cudaMemsetAsync(T.subVel, 0, sizeof(float4) * 8 * n, q));
    SPH_CUDA(cudaMemsetAsync(T.subAcc, 0, sizeof(float4) * 8 * n, q));
    SPH_CUDA(cudaMemsetAsync(T.subRho, 0, sizeof(float2) * 8 * n, q));
    SPH_CUDA(cudaMemsetAsync(T.subCnt, 0, sizeof(int) * (Cs + 1 + SCAN_TILE), q));
    SPH_CUDA(cudaMemsetAsync(T.subOffset, 0, sizeof(int) * (Cs + 1 + SCAN_TILE), q));
    for (int a = 0; a < 3; a++) {
        T.splitMin[a] = s->O.splitMin[a];
        T.splitMax[a] = s->O.splitMax[a];
    }
    T.childMode = s->O.childMode;
    s->subSb.cnt = T.subCnt;
    s->subSb.cellOffset = T.subOffset;
    s->subSb.tileCounter = reinterpret_cast<unsigned int*>(s->subScanBlock);
    s->subSb.scanFlags = s->subScanBlock + 2;
    s->subSb.maxTiles = (int)tiles;
    SPH_CUDA(cudaStreamSynchronize(q));
    s->tsReady = true;
    return SPH_OK;
}

// Enqueues one step of `mode` (no host synchronisation).
void request_list_build(sph_sim* s) {
    // every scene's VL_BUILD (any non-zero word requests)
    if (s->vlOn)
        cudaMemsetAsync(s->vl.flags + VL_BUILD * s->vl.numScenes, 1, sizeof(unsigned int) * s->vl.numScenes,
                        s->stream);
    s->lastStepLists = false;
}

// Before a sort outside the list steps: the cell tables it builds are current.
static void mark_tables_current(sph_sim* s) {
    if (s->vlOn)
        cudaMemsetAsync(s->vl.flags + VL_FLAGS * s->vl.numScenes + VL_STALE, 0, sizeof(unsigned int), s->stream);
}

void set_list_radius(sph_sim* s) {
    const float h = s->P.compactSupport, skin = s->O.neighbourSkin;
    s->vl.radius = (1.0f + skin) * h;
    s->vl.radius2 = s->vl.radius * s->vl.radius;
    const float lim = 0.45f * skin * h;
    s->vl.dispLimit2 = lim * lim;
    s->vl.skinFrac = skin;
}

sph_status alloc_lists(sph_sim* s) {
    if (!(s->O.neighbourSkin > 0.0f) || s->O.cellRelative) return SPH_OK;
    const size_t n = (size_t)s->n;
    const int S = std::max(s->numScenes, 1);
    SPH_CUDA(dalloc(&s->vl.start, VL_SLOTS * n));
    SPH_CUDA(dalloc(&s->vl.skin, VL_SLOTS * n));
    SPH_CUDA(dalloc(&s->vl.exact, VL_SLOTS * n));
    SPH_CUDA(dalloc(&s->vl.rows, n));
    SPH_CUDA(dalloc(&s->vl.posB, n));
    SPH_CUDA(dalloc(&s->vl.flags, (size_t)VL_FLAGS * S + VL_GLOBAL));
    SPH_CUDA(cudaMemsetAsync(s->vl.flags, 0, sizeof(unsigned int) * (VL_FLAGS * S + VL_GLOBAL), s->stream));
    s->vl.numScenes = S;
    if (S > 1) {  // each sorted slot's scene: scene k fills slots [sceneStart[k], sceneStart[k + 1])
        std::vector<int> scene(n);
        for (int k = 0; k < S; k++)
            std::fill(scene.begin() + s->sceneStart[(size_t)k], scene.begin() + s->sceneStart[(size_t)k + 1], k);
        SPH_CUDA(dalloc(&s->vl.slotScene, n));
        SPH_CUDA(cudaMemcpy(s->vl.slotScene, scene.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    }
    SPH_CUDA(cudaMemsetAsync(s->vl.rows, 0, n, s->stream));
    set_list_radius(s);
    s->vlOn = true;
    request_list_build(s);
    return SPH_OK;
}

// A plain step over the reused neighbour lists: the decision, the
// reference's hash, sort and cell tables when some scene builds (a step that
// builds nothing skips them; sph_read_cells builds its tables on demand),
// the state gathered into the lists' working order, then the density stage
// (building the lists when this step must) and the force stage over them.
static void enqueue_lists(sph_sim* s, const GridDev& g, const PhysDev& ph, int collide, cudaEvent_t* ev) {
    cudaStream_t st = s->stream;
    const int n = s->n;
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], st);
    };
    mark(ST_HASH);
    launch_hash_count(n, s->pos, g, s->sb, s->status, st, &s->vl);
    mark(ST_SCAN);
    launch_cell_scan(g.numCells, s->sb, s->status, st, &s->vl);
    mark(ST_SCATTER);
    launch_scatter(n, s->sb, st, s->status, &s->vl);
    mark(ST_RANK);
    launch_rank_gather(n, s->sb, s->pos, s->vel, g, s->posS, s->velS, st, &s->vl, s->status);
    mark(ST_DENSITY);
    launch_density_lists(n, s->posS, s->velS, rows_of(s), g, ph, s->map, s->rho4S, s->vl, s->cfg, true, true, st);
    // the sorted copies are now this step's own: a reuse the audit granted is used up
    cudaMemsetAsync(s->reuse, 0, sizeof(int), st);
    mark(ST_FORCE);
    launch_force_lists(n, s->posS, s->velS, s->rho4S, s->sb.workIds, ph, s->map, collide, s->vl, s->pos, s->vel,
                       s->accS, s->cfg, st, s->sb.scenes);
    mark(ST_FORCE + 1);  // the force stage's end
    s->lastStepLists = true;
}

void enqueue_coarse(sph_sim* s, const GridDev& g, const PhysDev& ph, int collide, cudaEvent_t* ev,
                    const FeatureOut* feat, bool force) {
    cudaStream_t st = s->stream;
    const int n = s->n;
    // the per-step search rewrites the sorted copies and the working order
    request_list_build(s);
    mark_tables_current(s);
    StepConfig cfg = s->cfg;
    // the feature form and the fused learned form read the density stage's masks
    if (feat || !force) cfg.forceVariant = FORCE_PRETESTED;
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], st);
    };
    mark(ST_HASH);
    launch_hash_count(n, s->pos, g, s->sb, s->status, st);
    mark(ST_SCAN);
    launch_cell_scan(g.numCells, s->sb, s->status, st);
    mark(ST_SCATTER);
    launch_scatter(n, s->sb, st, s->status);
    mark(ST_RANK);
    launch_rank_gather(n, s->sb, s->pos, s->vel, g, s->posS, s->velS, st, nullptr, s->status);
    mark(ST_DENSITY);
    // density and forces read the sorted copies only
    launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, cfg, st);
    // the sorted copies are now this step's own: a reuse the audit granted is used up
    cudaMemsetAsync(s->reuse, 0, sizeof(int), st);
    mark(ST_FORCE);
    if (!force) return;
    launch_force(n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), g, ph, s->map, collide, s->rowStart,
                 s->rowMask, s->pos, s->vel, s->accS, cfg, st, feat, s->status);
    mark(ST_FORCE + 1);  // the force stage's end
}

void enqueue_density_only(sph_sim* s, const float4* pos, const float4* vel, bool masks) {
    cudaStream_t st = s->stream;
    const int n = s->n;
    request_list_build(s);
    GridDev g = grid_of(s);
    PhysDev ph = make_phys(s->P, s->O);
    mark_tables_current(s);
    launch_hash_count(n, pos, g, s->sb, s->status, st);
    launch_cell_scan(g.numCells, s->sb, s->status, st);
    launch_scatter(n, s->sb, st, s->status);
    launch_rank_gather(n, s->sb, pos, vel, g, s->posS, s->velS, st, nullptr, s->status);
    StepConfig cfg = s->cfg;
    cfg.forceVariant = masks ? FORCE_PRETESTED : FORCE_MASK;  // whether to record the neighbour masks
    launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, cfg, st);
}

void enqueue_list_density(sph_sim* s, const float4* pos, const float4* vel) {
    cudaStream_t st = s->stream;
    const int n = s->n;
    GridDev g = grid_of(s);
    PhysDev ph = make_phys(s->P, s->O);
    launch_hash_count(n, pos, g, s->sb, s->status, st, &s->vl);
    launch_cell_scan(g.numCells, s->sb, s->status, st, &s->vl);
    launch_scatter(n, s->sb, st, s->status, &s->vl);
    launch_rank_gather(n, s->sb, pos, vel, g, s->posS, s->velS, st, &s->vl, s->status);
    launch_density_lists(n, s->posS, s->velS, rows_of(s), g, ph, s->map, s->rho4S, s->vl, s->cfg, true, true, st);
}

void invalidate_graphs(sph_sim* s) {
    s->graphValid = false;
    s->graphGen++;
}

void enqueue_step(sph_sim* s, int mode, bool timing, bool lists) {
    if (mode == SPH_STEP_SUB_ONLY) {
        if (!s->tsReady) return;
        // AdvanceSubParticles (:2119-2143) on the current lists
        cudaStream_t st = s->stream;
        const int cap = 8 * s->n;
        GridDev sg = make_grid(s->P, true);
        PhysDev sph = make_sub_phys(s->P, s->O);
        launch_ts_sub_sort(sg, s->ts, s->subSb, cap, s->status, st);
        launch_ts_sub_density(sg, sph, s->ts, cap, st);
        if (s->stepped)
            launch_ts_project(s->pos, s->sb.workIds, 1, s->rho4S, s->sb.cellOffset, make_grid(s->P, false),
                              s->P.compactSupportSub, s->ts, cap, st);
        launch_ts_sub_force(sg, sph, s->ts, cap, st);
        return;
    }
    const bool twoScale = mode == SPH_STEP_TWO_SCALE;
    cudaStream_t st = s->stream;
    const int n = s->n;
    GridDev g = grid_of(s);
    PhysDev ph = make_phys(s->P, s->O);
    cudaEvent_t* ev = nullptr;
    if (timing) {
        ev = &s->events[(size_t)s->timingNext * (ST_COUNT + 1)];
        // the stages this step runs (the events of the others are recorded at
        // its end, empty intervals that are not counted)
        s->timingRan[s->timingNext] = (1u << (twoScale ? ST_COUNT : ST_TS_CHILDREN)) - 1u;
        s->timingNext = (s->timingNext + 1) % s->timingCap;
        s->timingFilled = std::min(s->timingFilled + 1, s->timingCap);
    }
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], st);
    };
    auto mark_rest = [&](int k0) {
        for (int k = k0; k <= ST_COUNT; k++) mark(k);
    };
    // AdvanceTwoScale always runs handleCollisions (:2170)
    const int collide = twoScale ? 1 : s->O.boxCollision;
    if (!twoScale && lists && s->vlOn) {
        enqueue_lists(s, g, ph, collide, ev);
        mark_rest(ST_TS_CHILDREN + 1);
        return;
    }
    enqueue_coarse(s, g, ph, collide, ev);
    if (!twoScale) mark_rest(ST_TS_CHILDREN + 1);
    if (twoScale) {
        // computeParticleState, collect, initializeSubParticles, projectQuantities
        // (:2157-2160) from the pre-integration sorted state, which the force
        // stage leaves as it was (it writes the new state in particle order)
        launch_ts_states(n, s->posS, s->sb.workIds, s->sb.cellOffset, g, s->P.compactSupport, s->ts, st);
        launch_ts_children(n, s->posS, s->velS, s->accS, s->rho4S, s->sb.workIds, s->P.particleMass, ph, collide,
                           s->pos, s->vel, s->ts, st);
        launch_ts_project(s->posS, s->sb.workIds, 0, s->rho4S, s->sb.cellOffset, g, s->P.compactSupportSub,
                          s->ts, 8 * n, st);
        // the fine level (:2162-2171)
        const int cap = 8 * n;
        const GridDev sg = make_grid(s->P, true);
        PhysDev sph = make_sub_phys(s->P, s->O);
        mark(ST_SUB_SORT);
        launch_ts_sub_sort(sg, s->ts, s->subSb, cap, s->status, st);
        mark(ST_SUB_DENSITY);
        launch_ts_sub_density(sg, sph, s->ts, cap, st);
        mark(ST_SUB_FORCE);
        launch_ts_sub_force(sg, sph, s->ts, cap, st);
        mark(ST_COUNT);
    }
}

sph_status alloc_handle(sph_sim* s, int n, long long C) {
    s->n = n;
    s->numCellsTotal = C;
    const long long tiles = (C + 1 + SCAN_TILE - 1) / SCAN_TILE;
    SPH_CUDA(cudaGetDevice(&s->device));
    SPH_CUDA(cudaStreamCreateWithFlags(&s->ownStream, cudaStreamNonBlocking));
    s->stream = s->ownStream;
    SPH_CUDA(dalloc(&s->pos, n));
    SPH_CUDA(dalloc(&s->vel, n));
    SPH_CUDA(dalloc(&s->posS, n));
    SPH_CUDA(dalloc(&s->velS, n));
    SPH_CUDA(dalloc(&s->rho4S, n));
    SPH_CUDA(dalloc(&s->accS, n));
    SPH_CUDA(dalloc(&s->rowStart, (size_t)9 * n));
    SPH_CUDA(dalloc(&s->rowMask, (size_t)9 * n));
    SPH_CUDA(dalloc(&s->sb.cnt, (size_t)C + 1 + SCAN_TILE));
    SPH_CUDA(dalloc(&s->sb.cellOffset, (size_t)C + 1 + SCAN_TILE));
    SPH_CUDA(dalloc(&s->sb.keySlot, n));
    SPH_CUDA(dalloc(&s->sb.tmpIds, n));
    SPH_CUDA(dalloc(&s->sb.sortedHash, n));
    SPH_CUDA(dalloc(&s->sb.sortedIds, n));
    SPH_CUDA(dalloc(&s->sb.workIds, n));
    SPH_CUDA(dalloc(&s->sb.halfOffset, (size_t)C + 1));
    SPH_CUDA(cudaMemsetAsync(s->sb.halfOffset, 0, sizeof(int) * ((size_t)C + 1), s->stream));
    // index buffers start valid (0): an entry a failed step leaves unwritten
    // still names a particle or a cell of the handle
    for (int* p : {s->sb.tmpIds, s->sb.sortedHash, s->sb.sortedIds, s->sb.workIds})
        SPH_CUDA(cudaMemsetAsync(p, 0, sizeof(int) * (size_t)n, s->stream));
    SPH_CUDA(dalloc(&s->scanBlock, (size_t)tiles + 2));
    s->sb.tileCounter = reinterpret_cast<unsigned int*>(s->scanBlock);
    s->sb.scanFlags = s->scanBlock + 2;
    s->sb.maxTiles = (int)tiles;
    SPH_CUDA(dalloc(&s->status, 1));
    SPH_CUDA(dalloc(&s->reuse, 1));
    s->sb.skip = s->reuse;
    SPH_CUDA(cudaMallocHost((void**)&s->statusHost, sizeof(unsigned int)));
    SPH_CUDA(dalloc(&s->staging, (size_t)n * 10));
    SPH_CUDA(cudaMemsetAsync(s->sb.cnt, 0, sizeof(int) * ((size_t)C + 1 + SCAN_TILE), s->stream));
    SPH_CUDA(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->stream));
    SPH_CUDA(cudaMemsetAsync(s->reuse, 0, sizeof(int), s->stream));
    SPH_CUDA(cudaMemsetAsync(s->vel, 0, sizeof(float4) * n, s->stream));
    SPH_CUDA(cudaMemsetAsync(s->rho4S, 0, sizeof(float4) * n, s->stream));
    SPH_CUDA(cudaMemsetAsync(s->posS, 0, sizeof(float4) * n, s->stream));
    SPH_CUDA(cudaMemsetAsync(s->velS, 0, sizeof(float4) * n, s->stream));
    SPH_CUDA(cudaMemsetAsync(s->accS, 0, sizeof(float4) * n, s->stream));
    s->sdMass.assign(n, 0.0f);
    s->sdEnergy.assign(n, 0.0f);
    return SPH_OK;
}

MapDev map_of(const sph_boundary_desc& d, const unsigned int dims[3], const float4* map4, const float* dist) {
    MapDev m{};
    m.map4 = map4;
    m.dist = dist;
    for (int a = 0; a < 3; a++) {
        m.origin[a] = d.gridStart[a];
        m.dims[a] = (int)dims[a];
        m.dimsf[a] = (float)dims[a];
        m.length[a] = (float)(dims[a] - 1) * d.gridSpacing;
        m.du[a] = d.gridSpacing / m.length[a];
    }
    m.restDistance = d.restDistance;
    m.present = 1;
    return m;
}

GridDev grid_of(const sph_sim* s) {
    GridDev g = make_grid(s->P, false);
    g.numCells = (int)s->numCellsTotal;
    g.rel = s->O.cellRelative;
    return g;
}

// Each latched condition is reported once: the word is cleared when it is
// read back non-zero (a condition that persists, such as a particle still
// outside the grid, is latched again by the next step).
sph_status latched_status(sph_sim* s) {
    SPH_CUDA(cudaMemcpyAsync(s->statusHost, s->status, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                             s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    if (*s->statusHost) SPH_CUDA(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->stream));
    return status_of_host_copy(s);
}

sph_status status_of_host_copy(const sph_sim* s) {
    unsigned int v = *s->statusHost;
    if (v & STATUS_NON_FINITE) SPH_FAIL(SPH_ERR_NON_FINITE, "a non-finite particle position entered the step");
    if (v & STATUS_OUT_OF_DOMAIN)
        SPH_FAIL(SPH_ERR_OUT_OF_DOMAIN, "a particle was hashed outside the cell grid");
    if (v & STATUS_DEVICE_WAIT) SPH_FAIL(SPH_ERR_DEVICE_WAIT, "a bounded device-side wait gave up");
    return SPH_OK;
}

}  // namespace sph

extern "C" {

void sph_default_options(sph_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->gravityAxis = 1;
    o->boxCollision = 0;
    o->splitMin[0] = 0.2f;
    o->splitMax[0] = 0.5f;
    for (int a = 1; a < 3; a++) {
        o->splitMin[a] = -3.0e38f;
        o->splitMax[a] = 3.0e38f;
    }
    o->neighbourSkin = 0.1f;
}

const char* sph_last_error(void) { return g_lastError.c_str(); }

const char* sph_status_string(sph_status s) {
    switch (s) {
        case SPH_OK: return "ok";
        case SPH_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SPH_ERR_CUDA: return "CUDA error";
        case SPH_ERR_OUT_OF_MEMORY: return "out of device memory";
        case SPH_ERR_OUT_OF_DOMAIN: return "particle outside the cell grid";
        case SPH_ERR_DEVICE_WAIT: return "device-side wait gave up";
        case SPH_ERR_NOT_SUPPORTED: return "not supported";
        case SPH_ERR_NON_FINITE: return "non-finite particle position";
    }
    return "unknown status";
}

const char* sph_stage_name(int stage) {
    return stage >= 0 && stage < ST_COUNT ? kStageNames[stage] : "";
}

sph_status sph_boundary_dims(const sph_boundary_desc* desc, unsigned int dims[3]) {
    if (!dims) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "dims is NULL");
    return check_desc(desc, dims);
}

sph_status sph_boundary_maps(const sph_boundary_desc* desc, float* distance, float* density,
                             float* viscosity) {
    unsigned int dims[3];
    sph_status st = check_desc(desc, dims);
    if (st) return st;
    size_t total = (size_t)dims[0] * dims[1] * dims[2];
    float *d = nullptr, *r = nullptr, *v = nullptr;
    SPH_CUDA(dalloc(&d, total));
    cudaError_t e1 = dalloc(&r, total), e2 = dalloc(&v, total);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        cudaFree(d);
        if (r) cudaFree(r);
        if (v) cudaFree(v);
        SPH_FAIL(SPH_ERR_OUT_OF_MEMORY, "boundary map allocation failed");
    }
    cudaError_t e = launch_build_maps(*desc, dims, d, r, v, nullptr, 0);
    if (e == cudaSuccess && distance) e = cudaMemcpy(distance, d, total * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && density) e = cudaMemcpy(density, r, total * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && viscosity) e = cudaMemcpy(viscosity, v, total * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d);
    cudaFree(r);
    cudaFree(v);
    SPH_CUDA(e);
    return SPH_OK;
}

sph_status sph_create(const SimulationParameters* params, const sph_options* opts, const float* vertexData,
                      const float* simulationData, const sph_boundary_desc* boundary, sph_handle* out) {
    if (!out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    sph_status st = validate_params(params, opts);
    if (st) return st;
    if (!vertexData) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "vertexData is NULL");
    unsigned int mdims[3] = {0, 0, 0};
    if (boundary) {
        st = check_desc(boundary, mdims);
        if (st) return st;
    }
    sph_sim* s = new (std::nothrow) sph_sim();
    if (!s) SPH_FAIL(SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->P = *params;
    if (opts) s->O = *opts;
    else sph_default_options(&s->O);
    const int n = (int)params->numParticles;
    const long long C = (long long)params->gridDim[0] * params->gridDim[1] * params->gridDim[2];
    st = alloc_handle(s, n, C);
    if (!st) st = alloc_lists(s);
    if (st) {
        free_all(s);
        delete s;
        return st;
    }

#define CREATE_CUDA(call)                                                  \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            free_all(s);                                                   \
            delete s;                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA, \
                        __FILE__, __LINE__, cudaGetErrorString(e_));       \
        }                                                                  \
    } while (0)

    // initial state: VD positions, SD velocities
    CREATE_CUDA(cudaMemcpyAsync(s->staging, vertexData, sizeof(float) * 3 * (size_t)n,
                                cudaMemcpyHostToDevice, s->stream));
    launch_unpack_aos(s->staging, 3, 0, n, s->pos, s->stream);
    if (s->O.cellRelative) launch_abs_to_rel(n, s->pos, grid_of(s), s->stream);
    if (simulationData) {
        CREATE_CUDA(cudaStreamSynchronize(s->stream));
        CREATE_CUDA(cudaMemcpyAsync(s->staging, simulationData, sizeof(float) * 10 * (size_t)n,
                                    cudaMemcpyHostToDevice, s->stream));
        launch_unpack_aos(s->staging, 10, 6, n, s->vel, s->stream);
        for (int i = 0; i < n; i++) {
            s->sdMass[i] = simulationData[(size_t)i * 10 + 0];
            s->sdEnergy[i] = simulationData[(size_t)i * 10 + 9];
        }
    }
    if (boundary) {
        size_t total = (size_t)mdims[0] * mdims[1] * mdims[2];
        CREATE_CUDA(dalloc(&s->map4, total));
        CREATE_CUDA(dalloc(&s->mapDist, total));
        CREATE_CUDA(launch_build_maps(*boundary, mdims, s->mapDist, nullptr, nullptr, s->map4, s->stream));
        s->map = map_of(*boundary, mdims, s->map4, s->mapDist);
    }
    CREATE_CUDA(cudaGetLastError());
    CREATE_CUDA(cudaStreamSynchronize(s->stream));
#undef CREATE_CUDA
    *out = s;
    return SPH_OK;
}

sph_status sph_destroy(sph_handle s) {
    if (!s) return SPH_OK;
    cudaStreamSynchronize(s->stream);
    if (s->downStream) cudaStreamSynchronize(s->downStream);
    free_all(s);
    delete s;
    return SPH_OK;
}

sph_status sph_bind(sph_handle s, const SimulationParameters* params) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (s->numScenes > 1) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "batched handles keep their scenes' parameters");
    sph_status st = validate_params(params, &s->O);
    if (st) return st;
    if (params->numParticles != s->P.numParticles)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "numParticles cannot change after Init");
    for (int a = 0; a < 3; a++)
        if (params->gridDim[a] != s->P.gridDim[a] ||
            params->gridDimSubParticles[a] != s->P.gridDimSubParticles[a])
            SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "grid dimensions cannot change after Init");
    if (s->O.cellRelative) {
        // positions are relative to the grid: carry them over to the new one
        SPH_CUDA(cudaStreamSynchronize(s->stream));
        float4* tmp = nullptr;
        SPH_CUDA(dalloc(&tmp, (size_t)s->n));
        GridDev g0 = grid_of(s);
        SimulationParameters keep = s->P;
        s->P = *params;
        GridDev g1 = grid_of(s);
        s->P = keep;
        launch_rel_to_abs(s->n, s->pos, g0, nullptr, 0, tmp, s->stream);
        launch_abs_to_rel(s->n, tmp, g1, s->stream);
        cudaError_t e = cudaMemcpyAsync(s->pos, tmp, sizeof(float4) * (size_t)s->n, cudaMemcpyDeviceToDevice,
                                        s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        cudaFree(tmp);
        SPH_CUDA(e);
    }
    SPH_CUDA(cudaMemsetAsync(s->reuse, 0, sizeof(int), s->stream));
    s->P = *params;
    if (s->vlOn) set_list_radius(s);
    request_list_build(s);
    invalidate_graphs(s);
    return SPH_OK;
}

sph_status sph_set_stream(sph_handle s, void* stream) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    s->stream = stream ? (cudaStream_t)stream : s->ownStream;
    invalidate_graphs(s);
    return SPH_OK;
}

sph_status sph_step(sph_handle s, int mode) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (mode < SPH_STEP_PLAIN || mode > SPH_STEP_LEARNED) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown step mode");
    if (s->numScenes > 1 && mode != SPH_STEP_PLAIN)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "batched handles take plain steps only");
    if (s->O.cellRelative && mode != SPH_STEP_PLAIN)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "cell-relative positions take plain steps only");
    if (mode == SPH_STEP_LEARNED) return corrector_step(s, 1, false);
    if (mode != SPH_STEP_PLAIN) {
        sph_status st = ensure_two_scale(s);
        if (st) return st;
    }
    // a step graph captured by sph_step_many for this mode replays as one launch
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SPH_CUDA(cudaStreamIsCapturing(s->stream, &cs));
    if (s->timingCap == 0 && s->graphValid && s->graphMode == mode && mode != SPH_STEP_SUB_ONLY &&
        cs == cudaStreamCaptureStatusNone)
        SPH_CUDA(cudaGraphLaunch(s->graphExec, s->stream));
    else
        enqueue_step(s, mode, mode != SPH_STEP_SUB_ONLY && s->timingCap > 0);
    SPH_CUDA(cudaGetLastError());
    if (mode != SPH_STEP_SUB_ONLY) {
        s->numTimeSteps++;
        s->stepped = true;
        // whether the sorted copies match the lists (a replayed graph runs no
        // host code, so this is set here and not only where the work is enqueued)
        s->lastStepLists = mode == SPH_STEP_PLAIN && s->vlOn;
    }
    return SPH_OK;
}

sph_status sph_step_many(sph_handle s, int mode, int count) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (mode < SPH_STEP_PLAIN || mode > SPH_STEP_LEARNED) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown step mode");
    if (count <= 0) return SPH_OK;
    if (s->numScenes > 1 && mode != SPH_STEP_PLAIN)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "batched handles take plain steps only");
    if (s->O.cellRelative && mode != SPH_STEP_PLAIN)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "cell-relative positions take plain steps only");
    if (mode == SPH_STEP_LEARNED) return corrector_step(s, count, true);
    if (mode != SPH_STEP_PLAIN) {
        sph_status st = ensure_two_scale(s);
        if (st) return st;
    }
    if (mode == SPH_STEP_SUB_ONLY && !s->stepped) {
        for (int i = 0; i < count; i++) enqueue_step(s, mode, false);
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }
    if (s->graphMode != mode) s->graphValid = false;
    if (s->timingCap > 0) {
        for (int i = 0; i < count; i++) {
            sph_status st = sph_step(s, mode);
            if (st) return st;
        }
        return SPH_OK;
    }
    if (!s->graphValid) {
        if (s->graphExec) cudaGraphExecDestroy(s->graphExec);
        if (s->graph) cudaGraphDestroy(s->graph);
        s->graphExec = nullptr;
        s->graph = nullptr;
        SPH_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(s, mode, false);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        SPH_CUDA(e);
        s->graph = g;
        SPH_CUDA(cudaGraphInstantiate(&s->graphExec, s->graph, 0));
        s->graphValid = true;
        s->graphMode = mode;
    }
    for (int i = 0; i < count; i++) SPH_CUDA(cudaGraphLaunch(s->graphExec, s->stream));
    if (mode != SPH_STEP_SUB_ONLY) {
        s->numTimeSteps += (unsigned int)count;
        s->stepped = true;
        s->lastStepLists = mode == SPH_STEP_PLAIN && s->vlOn;
    }
    return SPH_OK;
}

sph_status sph_synchronize(sph_handle s) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    sph_status st = latched_status(s);
    // asynchronous reads finish on the side stream
    if (s->downStream) SPH_CUDA(cudaStreamSynchronize(s->downStream));
    return st;
}

namespace {

// Device-side two-scale counts: split, boundary, default, children.
sph_status two_scale_counts(sph_sim* s, int out[4]) {
    out[0] = out[1] = out[3] = 0;
    out[2] = s->n;
    if (!s->tsReady) return SPH_OK;
    SPH_CUDA(cudaMemcpyAsync(out, s->ts.counts, sizeof(int) * 4, cudaMemcpyDeviceToHost, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    return SPH_OK;
}

// Fields of the two-scale pass (states, lists, child slots).
sph_status read_two_scale(sph_sim* s, int field, void* dst, size_t bytes) {
    const size_t n = (size_t)s->n;
    int c[4];
    sph_status st = two_scale_counts(s, c);
    if (st) return st;
    cudaStream_t q = s->stream;
    size_t need = 0;
    const void* src = nullptr;
    switch (field) {
        case SPH_FIELD_STATE: need = n; src = s->ts.state; break;
        case SPH_FIELD_SUB_IDS: need = sizeof(int) * (size_t)c[3]; src = s->ts.subIds; break;
        case SPH_FIELD_SPLIT_IDS: need = sizeof(int) * (size_t)c[0]; src = s->ts.splitIds; break;
        case SPH_FIELD_BOUNDARY_IDS: need = sizeof(int) * (size_t)c[1]; src = s->ts.boundaryIds; break;
        case SPH_FIELD_DEFAULT_IDS: need = sizeof(int) * (size_t)c[2]; src = s->ts.defaultIds; break;
        case SPH_FIELD_SUB_VERTEX_DATA: need = sizeof(float) * 3 * 8 * n; break;
        case SPH_FIELD_SUB_SIMULATION_DATA: need = sizeof(float) * 10 * 8 * n; break;
    }
    if (bytes < need) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "destination too small");
    if (!s->tsReady) {
        // before any two-scale step: every particle is in the default state
        if (field == SPH_FIELD_DEFAULT_IDS)
            for (size_t i = 0; i < n; i++) static_cast<int*>(dst)[i] = (int)i;
        else std::memset(dst, 0, need);
        return SPH_OK;
    }
    if (src) {
        if (need) SPH_CUDA(cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToHost, q));
        SPH_CUDA(cudaStreamSynchronize(q));
        return SPH_OK;
    }
    float* tmp = nullptr;
    SPH_CUDA(cudaMalloc((void**)&tmp, need));
    if (field == SPH_FIELD_SUB_VERTEX_DATA) launch_pack_aos(s->ts.subPos, (int)(8 * n), tmp, 3, 0, q);
    else launch_ts_pack_sd(s->ts, (int)(8 * n), tmp, q);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, tmp, need, cudaMemcpyDeviceToHost, q);
    if (e == cudaSuccess) e = cudaStreamSynchronize(q);
    cudaFree(tmp);
    SPH_CUDA(e);
    return SPH_OK;
}

}  // namespace

// Whether the stream has queued work that has not finished (not while it is
// being captured: a captured stream takes the plain path).
static bool stream_busy(cudaStream_t q) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(q, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
    const cudaError_t e = cudaStreamQuery(q);
    if (e == cudaErrorNotReady) {
        cudaGetLastError();  // (not an error: clear it)
        return true;
    }
    return false;
}

// The side streams, their buffers and events, made on first use (all or
// nothing).
static cudaError_t ensure_side_streams(sph_sim* s) {
    if (s->upStream) return cudaSuccess;
    const size_t n3 = 3 * (size_t)s->n;
    cudaStream_t up = nullptr, down = nullptr;
    float *land[2] = {nullptr, nullptr}, *stage = nullptr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaError_t e = cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = dalloc(&land[k], n3);
    if (e == cudaSuccess) e = dalloc(&stage, n3);
    for (int k = 0; k < 6 && e == cudaSuccess; k++) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        for (float* p : {land[0], land[1], stage})
            if (p) cudaFree(p);
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        for (cudaStream_t q : {up, down})
            if (q) cudaStreamDestroy(q);
        return e;
    }
    s->upStream = up;
    s->downStream = down;
    for (int k = 0; k < 2; k++) {
        s->upLand[k] = land[k];
        s->upReady[k] = ev[k];
        s->upFree[k] = ev[2 + k];
    }
    s->downStage = stage;
    s->downReady = ev[4];
    s->downFree = ev[5];
    return cudaSuccess;
}

// The fields of the particle grid; `wait`: return when the data is there
// and report the latched conditions, else only enqueue (no host-side step).
static sph_status read_field(sph_sim* s, int field, void* dst, size_t bytes, bool wait) {
    const int n = s->n;
    size_t need = 0;
    switch (field) {
        case SPH_FIELD_VERTEX_DATA:
        case SPH_FIELD_VELOCITY:
        case SPH_FIELD_ACCELERATION: need = sizeof(float) * 3 * (size_t)n; break;
        case SPH_FIELD_SIMULATION_DATA: need = sizeof(float) * 10 * (size_t)n; break;
        case SPH_FIELD_DENSITY:
        case SPH_FIELD_PRESSURE: need = sizeof(float) * (size_t)n; break;
        default: SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown field");
    }
    if (bytes < need) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "destination too small");
    cudaStream_t q = s->stream;
    // positions and velocities bound for page-locked memory are packed by the
    // kernel straight into it over the host link (12 MB: 68 us, against 80 us
    // for a pack into device memory and a DMA copy); the other fields and
    // pageable destinations go through the staging buffer and one DMA copy
    float* direct = nullptr;
    if (wait && ((field == SPH_FIELD_VERTEX_DATA && !s->O.cellRelative) || field == SPH_FIELD_VELOCITY))
        direct = static_cast<float*>(host_device_ptr(dst));
    float* out = direct ? direct : s->staging;
    if (!wait) {
        // packed on the handle's stream into a buffer of its own, copied to
        // the host by DMA on the side stream: the next step need not wait
        SPH_CUDA(ensure_side_streams(s));
        SPH_CUDA(cudaStreamWaitEvent(q, s->downFree, 0));
        out = s->downStage;
    }
    switch (field) {
        case SPH_FIELD_VERTEX_DATA:
            if (s->O.cellRelative) launch_rel_to_abs(n, s->pos, grid_of(s), out, 3, nullptr, q);
            else launch_pack_aos(s->pos, n, out, 3, 0, q);
            break;
        case SPH_FIELD_VELOCITY: launch_pack_aos(s->vel, n, out, 3, 0, q); break;
        case SPH_FIELD_ACCELERATION:
            if (s->stepped) launch_unpermute(n, s->sb.workIds, s->accS, -1, out, 3, 0, q);
            else SPH_CUDA(cudaMemsetAsync(out, 0, need, q));
            break;
        case SPH_FIELD_DENSITY:
        case SPH_FIELD_PRESSURE:
            if (s->stepped)
                launch_unpermute(n, s->sb.workIds, s->rho4S, field == SPH_FIELD_DENSITY ? 0 : 1, out, 1, 0, q);
            else SPH_CUDA(cudaMemsetAsync(out, 0, need, q));
            break;
        case SPH_FIELD_SIMULATION_DATA:
            SPH_CUDA(cudaMemsetAsync(out, 0, need, q));
            if (s->stepped) {
                launch_unpermute(n, s->sb.workIds, s->rho4S, 0, out, 10, 1, q);
                launch_unpermute(n, s->sb.workIds, s->rho4S, 1, out, 10, 2, q);
                launch_unpermute(n, s->sb.workIds, s->accS, -1, out, 10, 3, q);
            }
            launch_pack_aos(s->vel, n, out, 10, 6, q);
            break;
    }
    SPH_CUDA(cudaGetLastError());
    if (!wait) {
        SPH_CUDA(cudaEventRecord(s->downReady, q));
        SPH_CUDA(cudaStreamWaitEvent(s->downStream, s->downReady, 0));
        SPH_CUDA(cudaMemcpyAsync(dst, s->downStage, need, cudaMemcpyDeviceToHost, s->downStream));
        SPH_CUDA(cudaEventRecord(s->downFree, s->downStream));
        return SPH_OK;
    }
    if (!direct) SPH_CUDA(cudaMemcpyAsync(dst, s->staging, need, cudaMemcpyDeviceToHost, q));
    // one synchronisation: the status word comes back with the data
    SPH_CUDA(cudaMemcpyAsync(s->statusHost, s->status, sizeof(unsigned int), cudaMemcpyDeviceToHost, q));
    SPH_CUDA(cudaStreamSynchronize(q));
    if (*s->statusHost) SPH_CUDA(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), q));  // reported once
    sph_status st = status_of_host_copy(s);
    if (st) return st;
    if (field == SPH_FIELD_SIMULATION_DATA) {
        float* f = static_cast<float*>(dst);
        for (int i = 0; i < n; i++) {
            f[(size_t)i * 10 + 0] = s->sdMass[i];
            f[(size_t)i * 10 + 9] = s->sdEnergy[i];
        }
    }
    return SPH_OK;
}

sph_status sph_read(sph_handle s, int field, void* dst, size_t bytes) {
    if (!s || !dst) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (field == SPH_FIELD_STATE || (field >= SPH_FIELD_SUB_VERTEX_DATA && field <= SPH_FIELD_DEFAULT_IDS)) {
        sph_status st = latched_status(s);
        if (st) return st;
        return read_two_scale(s, field, dst, bytes);
    }
    return read_field(s, field, dst, bytes, true);
}

sph_status sph_read_async(sph_handle s, int field, void* dst, size_t bytes) {
    if (!s || !dst) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (field < SPH_FIELD_VERTEX_DATA || field > SPH_FIELD_PRESSURE || field == SPH_FIELD_SIMULATION_DATA)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "sph_read_async takes VD, velocity, acceleration, density or pressure");
    return read_field(s, field, dst, bytes, false);
}

sph_status sph_write(sph_handle s, int field, const void* src, size_t bytes) {
    if (!s || !src) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    const int n = s->n;
    cudaStream_t q = s->stream;
    SPH_CUDA(cudaMemsetAsync(s->reuse, 0, sizeof(int), q));  // the state changes under the sorted copies
    switch (field) {
        case SPH_FIELD_VERTEX_DATA:
        case SPH_FIELD_VELOCITY: {
            if (bytes < sizeof(float) * 3 * (size_t)n) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "source too small");
            // page-locked sources are read by the unpacking kernel itself
            const float* in = static_cast<const float*>(host_device_ptr(src));
            float4* target = field == SPH_FIELD_VERTEX_DATA ? s->pos : s->vel;
            if (!in) {
                SPH_CUDA(cudaMemcpyAsync(s->staging, src, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, q));
                launch_unpack_aos(s->staging, 3, 0, n, target, q);
            } else if (stream_busy(q)) {
                // the handle's stream still has work: a DMA copy on the side
                // stream lands the data beside that work (the copy engines,
                // not the SMs the queued kernels hold), and the handle's stream
                // unpacks it into place once it has landed
                SPH_CUDA(ensure_side_streams(s));
                const int k = field == SPH_FIELD_VERTEX_DATA ? 0 : 1;
                SPH_CUDA(cudaStreamWaitEvent(s->upStream, s->upFree[k], 0));
                SPH_CUDA(cudaMemcpyAsync(s->upLand[k], src, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice,
                                         s->upStream));
                SPH_CUDA(cudaEventRecord(s->upReady[k], s->upStream));
                SPH_CUDA(cudaStreamWaitEvent(q, s->upReady[k], 0));
                launch_unpack_aos(s->upLand[k], 3, 0, n, target, q);
                SPH_CUDA(cudaEventRecord(s->upFree[k], q));
            } else {
                launch_unpack_aos(in, 3, 0, n, target, q);
            }
            if (field == SPH_FIELD_VERTEX_DATA && s->O.cellRelative) launch_abs_to_rel(n, s->pos, grid_of(s), q);
            if (field == SPH_FIELD_VERTEX_DATA && s->numScenes > 1)  // restore the scene index lanes
                for (int k = 0; k < s->numScenes; k++)
                    launch_set_scene(s->pos + s->sceneStart[k], (int)(s->sceneStart[k + 1] - s->sceneStart[k]), k, q);
            // the lists stay valid while every particle is within the rebuild
            // distance of where it was at their build (velocities do not matter)
            if (field == SPH_FIELD_VERTEX_DATA && s->vlOn && s->lastStepLists)
                launch_list_displacement(n, s->pos, s->sb.workIds, s->vl, q);
            break;
        }
        case SPH_FIELD_SIMULATION_DATA:
            if (bytes < sizeof(float) * 10 * (size_t)n) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "source too small");
            SPH_CUDA(cudaMemcpyAsync(s->staging, src, sizeof(float) * 10 * (size_t)n, cudaMemcpyHostToDevice, q));
            launch_unpack_aos(s->staging, 10, 6, n, s->vel, q);
            for (int i = 0; i < n; i++) {
                s->sdMass[i] = static_cast<const float*>(src)[(size_t)i * 10 + 0];
                s->sdEnergy[i] = static_cast<const float*>(src)[(size_t)i * 10 + 9];
            }
            break;
        default: SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "field is not writable");
    }
    SPH_CUDA(cudaGetLastError());
    return SPH_OK;
}

sph_status sph_read_cells(sph_handle s, int level, int* sortedHash, int* sortedIds, int* cellStart,
                          int* cellEnd) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (level != 0 && level != 1) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "level must be 0 or 1");
    if (!s->stepped) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no step has run yet");
    sph_status st = latched_status(s);
    if (st) return st;
    if (level == 1) {
        // the fine level of the last two-scale step: arrays of numSubParticles
        if (!s->tsReady) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no two-scale step has run yet");
        int c[4];
        st = two_scale_counts(s, c);
        if (st) return st;
        const int Cs = s->P.gridDimSubParticles[0] * s->P.gridDimSubParticles[1] * s->P.gridDimSubParticles[2];
        cudaStream_t q = s->stream;
        if (sortedHash && c[3])
            SPH_CUDA(cudaMemcpyAsync(sortedHash, s->ts.subSortedHash, sizeof(int) * c[3], cudaMemcpyDeviceToHost, q));
        if (sortedIds && c[3])
            SPH_CUDA(cudaMemcpyAsync(sortedIds, s->ts.subSortedIds, sizeof(int) * c[3], cudaMemcpyDeviceToHost, q));
        if (cellStart || cellEnd) {
            int* tmp = nullptr;
            SPH_CUDA(cudaMalloc((void**)&tmp, sizeof(int) * 2 * (size_t)Cs));
            if (c[3]) {
                launch_cell_tables(Cs, s->ts.subOffset, tmp, tmp + Cs, q);
            } else {
                cudaMemsetAsync(tmp, 0xFF, sizeof(int) * 2 * (size_t)Cs, q);
            }
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess && cellStart) e = cudaMemcpyAsync(cellStart, tmp, sizeof(int) * Cs, cudaMemcpyDeviceToHost, q);
            if (e == cudaSuccess && cellEnd) e = cudaMemcpyAsync(cellEnd, tmp + Cs, sizeof(int) * Cs, cudaMemcpyDeviceToHost, q);
            if (e == cudaSuccess) e = cudaStreamSynchronize(q);
            cudaFree(tmp);
            SPH_CUDA(e);
        }
        SPH_CUDA(cudaStreamSynchronize(q));
        return SPH_OK;
    }
    const int n = s->n;
    const int C = (int)s->numCellsTotal;
    cudaStream_t q = s->stream;
    if (s->vlOn) {
        // a step over the reused lists that built none skipped the tables:
        // built now from that step's sorted copies, as it would have built them
        unsigned int* stale = s->vl.flags + VL_FLAGS * s->vl.numScenes + VL_STALE;
        SPH_CUDA(cudaMemcpyAsync(s->statusHost, stale, sizeof(unsigned int), cudaMemcpyDeviceToHost, q));
        SPH_CUDA(cudaStreamSynchronize(q));
        if (*s->statusHost) {
            float4* scratch = nullptr;
            unsigned int* st2 = nullptr;
            cudaError_t e = dalloc(&scratch, (size_t)n);
            if (e == cudaSuccess) e = dalloc(&st2, 1);
            // the step reported its conditions already: the rebuild's go to a word of their own
            if (e == cudaSuccess) e = cudaMemsetAsync(st2, 0, sizeof(unsigned int), q);
            if (e == cudaSuccess) {
                launch_rebuild_tables(n, s->posS, s->sb.workIds, s->vl.slotScene, grid_of(s), s->sb, scratch, st2,
                                      q);
                e = cudaMemsetAsync(stale, 0, sizeof(unsigned int), q);
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(q);
            cudaFree(scratch);
            cudaFree(st2);
            SPH_CUDA(e);
        }
    }
    if (sortedHash)
        SPH_CUDA(cudaMemcpyAsync(sortedHash, s->sb.sortedHash, sizeof(int) * n, cudaMemcpyDeviceToHost, q));
    if (sortedIds)
        SPH_CUDA(cudaMemcpyAsync(sortedIds, s->sb.sortedIds, sizeof(int) * n, cudaMemcpyDeviceToHost, q));
    if (cellStart || cellEnd) {
        // the per-cell counters are zero between steps: borrow them as the
        // start/end staging area (2*C ints needed, C+1+tile available) in two rounds
        int* tmp = s->sb.cnt;
        if (cellStart) {
            launch_cell_tables(C, s->sb.cellOffset, tmp, nullptr, q);
            SPH_CUDA(cudaMemcpyAsync(cellStart, tmp, sizeof(int) * (size_t)C, cudaMemcpyDeviceToHost, q));
        }
        if (cellEnd) {
            launch_cell_tables(C, s->sb.cellOffset, nullptr, tmp, q);
            SPH_CUDA(cudaMemcpyAsync(cellEnd, tmp, sizeof(int) * (size_t)C, cudaMemcpyDeviceToHost, q));
        }
        SPH_CUDA(cudaMemsetAsync(tmp, 0, sizeof(int) * ((size_t)C + 1), q));
    }
    SPH_CUDA(cudaGetLastError());
    SPH_CUDA(cudaStreamSynchronize(q));
    return SPH_OK;
}

sph_status sph_get_counts(sph_handle s, sph_counts* out) {
    if (!s || !out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    int c[4];
    sph_status st = two_scale_counts(s, c);
    if (st) return st;
    out->numParticles = (unsigned int)s->n;
    out->numParticlesSplit = (unsigned int)c[0];
    out->numParticlesBoundary = (unsigned int)c[1];
    out->numParticlesDefault = (unsigned int)c[2];
    out->numSubParticles = (unsigned int)c[3];
    out->numTimeSteps = s->numTimeSteps;
    out->numCells = (unsigned int)s->numCellsTotal;
    out->numSubCells = (unsigned int)(s->P.gridDimSubParticles[0] * s->P.gridDimSubParticles[1] *
                                      s->P.gridDimSubParticles[2]);
    return SPH_OK;
}

sph_status sph_get_diagnostics(sph_handle s, sph_diagnostics* out) {
    if (!s || !out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (s->numScenes > 1) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "diagnostics are per scene: not for batched handles");
    const int rows = diag_partial_rows();
    if (!s->diagBuf) SPH_CUDA(dalloc(&s->diagBuf, (size_t)(rows + 1) * DIAG_TERMS));
    double* res = s->diagBuf + (size_t)rows * DIAG_TERMS;
    const float4* posAbs = s->pos;
    if (s->O.cellRelative) {  // the potential energy needs absolute heights: staging holds 10n floats
        launch_rel_to_abs(s->n, s->pos, grid_of(s), nullptr, 0, reinterpret_cast<float4*>(s->staging), s->stream);
        posAbs = reinterpret_cast<const float4*>(s->staging);
    }
    launch_diagnostics(s->n, posAbs, s->vel, s->rho4S, s->stepped ? 1 : 0, (double)s->P.particleMass,
                       (double)s->P.gravity, (double)s->P.restDensity, s->O.gravityAxis, s->diagBuf, res,
                       s->stream);
    SPH_CUDA(cudaGetLastError());
    double h[DIAG_TERMS];
    SPH_CUDA(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    sph_status st = latched_status(s);
    if (st) return st;
    out->mass = h[DIAG_MASS];
    out->momentum[0] = h[DIAG_MOM_X];
    out->momentum[1] = h[DIAG_MOM_Y];
    out->momentum[2] = h[DIAG_MOM_Z];
    out->kineticEnergy = h[DIAG_KINETIC];
    out->potentialEnergy = h[DIAG_POTENTIAL];
    out->densityMean = h[DIAG_RHO_SUM] / (double)s->n;
    out->densityMaxRelError = h[DIAG_RHO_MAXERR];
    return SPH_OK;
}

sph_status sph_device_pointer(sph_handle s, int which, void** devicePtr) {
    if (!s || !devicePtr) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (which == 0 && s->O.cellRelative)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "cell-relative positions are not absolute float4s: use sph_read");
    if (which == 0) *devicePtr = s->pos;
    else if (which == 1) *devicePtr = s->vel;
    else SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown device field");
    return SPH_OK;
}

sph_status sph_set_stage_timing(sph_handle s, int enable) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    s->events.clear();
    s->timingRan.clear();
    s->timingCap = s->timingNext = s->timingFilled = 0;
    if (enable > 0) {
        int cap = enable;
        s->events.resize((size_t)cap * (ST_COUNT + 1));
        for (auto& e : s->events) SPH_CUDA(cudaEventCreate(&e));
        s->timingRan.assign((size_t)cap, 0u);
        s->timingCap = cap;
    }
    return SPH_OK;
}

sph_status sph_get_tuning(sph_handle s, sph_tuning* out) {
    if (!s || !out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    out->densityBlock = s->cfg.densityBlock;
    out->forceBlock = s->cfg.forceBlock;
    out->forceVariant = s->cfg.forceVariant;
    out->prune = s->cfg.prune;
    out->kahan = s->cfg.kahan;
    return SPH_OK;
}

sph_status sph_set_tuning(sph_handle s, const sph_tuning* t) {
    if (!s || !t) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    auto okBlock = [](int b) { return b == 64 || b == 128 || b == 256; };
    if (!okBlock(t->densityBlock) || !okBlock(t->forceBlock))
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "block sizes must be 64, 128 or 256");
    if (t->forceVariant < FORCE_DIRECT || t->forceVariant > FORCE_STAGED)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "unknown force variant");
    s->cfg.densityBlock = t->densityBlock;
    s->cfg.forceBlock = t->forceBlock;
    s->cfg.forceVariant = t->forceVariant;
    s->cfg.prune = t->prune ? 1 : 0;
    s->cfg.kahan = t->kahan ? 1 : 0;
    invalidate_graphs(s);
    return SPH_OK;
}

// The autotuner of a handle with reused neighbour lists: the list kernels
// have one form each, so only their block sizes are tried, by whole steps
// from the current state.  The state, the sorted copies and tables, and the
// lists with their flags are saved first and put back afterwards, so the
// next step is the one that would have come without the tuning.
static sph_status autotune_lists(sph_sim* s, int reps, sph_tuning* chosen) {
    const int n = s->n;
    const size_t C1 = (size_t)s->numCellsTotal + 1;
    cudaStream_t st = s->stream;
    struct Buf {
        void* dst;
        void* save;
        size_t bytes;
    } bufs[] = {{s->pos, nullptr, sizeof(float4) * n},          {s->vel, nullptr, sizeof(float4) * n},
                {s->posS, nullptr, sizeof(float4) * n},         {s->velS, nullptr, sizeof(float4) * n},
                {s->rho4S, nullptr, sizeof(float4) * n},        {s->accS, nullptr, sizeof(float4) * n},
                {s->sb.sortedHash, nullptr, sizeof(int) * n},   {s->sb.sortedIds, nullptr, sizeof(int) * n},
                {s->sb.workIds, nullptr, sizeof(int) * n},      {s->sb.cellOffset, nullptr, sizeof(int) * C1},
                {s->sb.halfOffset, nullptr, sizeof(int) * C1},
                {s->vl.flags, nullptr, sizeof(unsigned int) * (VL_FLAGS * s->vl.numScenes + VL_GLOBAL)},
                {s->vl.start, nullptr, sizeof(int) * VL_SLOTS * n},
                {s->vl.skin, nullptr, sizeof(uint2) * VL_SLOTS * n},
                {s->vl.exact, nullptr, sizeof(uint2) * VL_SLOTS * n},
                {s->vl.rows, nullptr, (size_t)n},               {s->vl.posB, nullptr, sizeof(float4) * n}};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        for (auto& b : bufs)
            if (b.save) cudaFree(b.save);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t te = cudaStreamSynchronize(st);
    for (auto& b : bufs) {
        if (te == cudaSuccess) te = cudaMalloc(&b.save, b.bytes);
        if (te == cudaSuccess) te = cudaMemcpyAsync(b.save, b.dst, b.bytes, cudaMemcpyDeviceToDevice, st);
    }
    if (te == cudaSuccess) te = cudaEventCreate(&e0);
    if (te == cudaSuccess) te = cudaEventCreate(&e1);
    const unsigned int steps0 = s->numTimeSteps;
    const bool stepped0 = s->stepped;
    const bool lists0 = s->lastStepLists;
    const StepConfig current = s->cfg;
    std::vector<StepConfig> trials{current};
    for (int db : {64, 128, 256})
        for (int fb : {64, 128, 256}) {
            StepConfig c = current;
            c.densityBlock = db;
            c.forceBlock = fb;
            if (db != current.densityBlock || fb != current.forceBlock) trials.push_back(c);
        }
    float bestStep = 3.0e38f;
    StepConfig chosenCfg = current;
    for (size_t k = 0; k < trials.size() && te == cudaSuccess; k++) {
        s->cfg = trials[k];
        invalidate_graphs(s);
        float fastest = 3.0e38f;
        for (int r = 0; r < std::max(reps, 1) && te == cudaSuccess; r++) {
            te = cudaMemcpyAsync(s->pos, bufs[0].save, bufs[0].bytes, cudaMemcpyDeviceToDevice, st);
            if (te == cudaSuccess) te = cudaMemcpyAsync(s->vel, bufs[1].save, bufs[1].bytes, cudaMemcpyDeviceToDevice, st);
            request_list_build(s);
            // capture and the build step, then list steps only
            if (te == cudaSuccess && sph_step_many(s, SPH_STEP_PLAIN, 2) != SPH_OK) te = cudaErrorUnknown;
            if (te == cudaSuccess) te = cudaEventRecord(e0, st);
            if (te == cudaSuccess && sph_step_many(s, SPH_STEP_PLAIN, 8) != SPH_OK) te = cudaErrorUnknown;
            if (te == cudaSuccess) te = cudaEventRecord(e1, st);
            if (te == cudaSuccess) te = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
            if (te == cudaSuccess) fastest = std::min(fastest, ms);
        }
        // keep the incumbent unless beaten by 2 %
        if (te == cudaSuccess && fastest < (k == 0 ? bestStep : 0.98f * bestStep)) {
            bestStep = fastest;
            chosenCfg = trials[k];
        }
    }
    for (auto& b : bufs)
        if (te == cudaSuccess && b.save) te = cudaMemcpyAsync(b.dst, b.save, b.bytes, cudaMemcpyDeviceToDevice, st);
    if (te == cudaSuccess) te = cudaStreamSynchronize(st);
    cleanup();
    s->numTimeSteps = steps0;
    s->stepped = stepped0;
    s->cfg = te == cudaSuccess ? chosenCfg : current;
    // the lists, their flags and the sorted copies are as the last step left them
    s->lastStepLists = lists0;
    if (te != cudaSuccess) request_list_build(s);
    invalidate_graphs(s);
    SPH_CUDA(te);
    if (chosen) return sph_get_tuning(s, chosen);
    return SPH_OK;
}

sph_status sph_autotune(sph_handle s, int reps, sph_tuning* chosen) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    reps = std::max(reps, 1);
    if (s->vlOn) return autotune_lists(s, reps, chosen);
    const int n = s->n;
    const int C = (int)s->numCellsTotal;
    cudaStream_t st = s->stream;
    // the trials rewrite the sorted copies and masks: no step may reuse them
    SPH_CUDA(cudaMemsetAsync(s->reuse, 0, sizeof(int), st));
    SPH_CUDA(cudaStreamSynchronize(st));
    // keep the last step's sorted data (read-back) and write forces to scratch
    struct Buf {
        void* dst;
        void* save;
        size_t bytes;
    } bufs[] = {{s->posS, nullptr, sizeof(float4) * n},       {s->velS, nullptr, sizeof(float4) * n},
                {s->rho4S, nullptr, sizeof(float4) * n},      {s->sb.sortedHash, nullptr, sizeof(int) * n},
                {s->sb.sortedIds, nullptr, sizeof(int) * n},  {s->sb.cellOffset, nullptr, sizeof(int) * ((size_t)C + 1)},
                {s->sb.workIds, nullptr, sizeof(int) * n},    {s->accS, nullptr, sizeof(float4) * n},
                {s->sb.halfOffset, nullptr, sizeof(int) * ((size_t)C + 1)}};
    float4* scratch = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        for (auto& b : bufs)
            if (b.save) cudaFree(b.save);
        if (scratch) cudaFree(scratch);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
#define TUNE_CUDA(call)                                                                  \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            cleanup();                                                                   \
            return fail(SPH_ERR_CUDA, __FILE__, __LINE__, cudaGetErrorString(e_));       \
        }                                                                                \
    } while (0)
    for (auto& b : bufs) {
        TUNE_CUDA(cudaMalloc(&b.save, b.bytes));
        TUNE_CUDA(cudaMemcpyAsync(b.save, b.dst, b.bytes, cudaMemcpyDeviceToDevice, st));
    }
    TUNE_CUDA(cudaMalloc((void**)&scratch, sizeof(float4) * 3 * (size_t)n));
    TUNE_CUDA(cudaEventCreate(&e0));
    TUNE_CUDA(cudaEventCreate(&e1));
    GridDev g = grid_of(s);
    PhysDev ph = make_phys(s->P, s->O);
    auto sortStages = [&]() {
        launch_hash_count(n, s->pos, g, s->sb, s->status, st);
        launch_cell_scan(g.numCells, s->sb, s->status, st);
        launch_scatter(n, s->sb, st, s->status);
        launch_rank_gather(n, s->sb, s->pos, s->vel, g, s->posS, s->velS, st, nullptr, s->status);
    };
    // each candidate is timed in step context: the sort stages run before
    // every timed launch, so caches hold what they hold in a real step; the
    // fastest of the repeats counts (the least disturbed one)
    auto timeit = [&](auto&& before, auto&& launch) -> float {
        float fastest = 3.0e38f;
        for (int r = 0; r < reps + 1; r++) {
            before();
            cudaEventRecord(e0, st);
            launch();
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) fastest = std::min(fastest, ms);  // the first launch warms up
        }
        return fastest;
    };
    const int blocks[3] = {64, 128, 256};
    // the configuration in use is kept unless a candidate beats it by 2 %
    const StepConfig current = s->cfg;
    auto stepTime = [&](const StepConfig& c) {
        const float d = timeit(sortStages, [&] {
            launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, c, st);
        });
        const float f = timeit(
            [&] {
                sortStages();
                launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, c, st);
            },
            [&] {
                launch_force(n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), g, ph, s->map,
                             s->O.boxCollision, s->rowStart, s->rowMask, scratch, scratch + n,
                             scratch + 2 * (size_t)n, c, st, nullptr, s->status);
            });
        return d + f;
    };
    const float currentTotal = stepTime(current);
    StepConfig best = current;
    float bestTotal = currentTotal;
    std::vector<std::pair<float, StepConfig>> shapes;  // the best block sizes of each form and cut
    for (int prune = 0; prune <= 1; prune++)
        for (int v = FORCE_DIRECT; v <= FORCE_STAGED; v++) {
            StepConfig c = s->cfg;
            c.prune = prune;
            c.forceVariant = v;  // the density stage records masks for the pretested and staged forms
            float bestD = 3.0e38f;
            int bestDB = c.densityBlock;
            for (int b : blocks) {
                c.densityBlock = b;
                float t = timeit(sortStages, [&] {
                    launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, c, st);
                });
                if (t < bestD) {
                    bestD = t;
                    bestDB = b;
                }
            }
            c.densityBlock = bestDB;
            auto beforeForce = [&]() {
                sortStages();
                launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, c, st);
            };
            float bestF = 3.0e38f;
            StepConfig bestC = c;
            for (int b : blocks) {
                c.forceBlock = b;
                float t = timeit(beforeForce, [&] {
                    launch_force(n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), g, ph, s->map,
                                 s->O.boxCollision, s->rowStart, s->rowMask, scratch, scratch + n,
                                 scratch + 2 * (size_t)n, c, st, nullptr, s->status);
                });
                if (t < bestF) {
                    bestF = t;
                    bestC = c;
                }
                if (bestD + t < bestTotal) {
                    bestTotal = bestD + t;
                    best = c;
                }
            }
            shapes.push_back({bestD + bestF, bestC});
        }
    if (bestTotal > 0.98f * currentTotal) best = current;
    TUNE_CUDA(cudaGetLastError());
    for (auto& b : bufs) TUNE_CUDA(cudaMemcpyAsync(b.dst, b.save, b.bytes, cudaMemcpyDeviceToDevice, st));
    TUNE_CUDA(cudaStreamSynchronize(st));

    // Whole steps decide between the leading shapes: the stage estimates miss
    // how the stages share the caches and overlap inside a step graph.  The
    // particle state is saved and put back around each trial.
    std::sort(shapes.begin(), shapes.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    // the configuration in use is the incumbent
    std::vector<StepConfig> finalists{current, best};
    for (size_t k = 0; k < shapes.size() && finalists.size() < 5; k++) finalists.push_back(shapes[k].second);
    float4 *savePos = nullptr, *saveVel = nullptr;
    TUNE_CUDA(cudaMalloc((void**)&savePos, sizeof(float4) * n));
    TUNE_CUDA(cudaMalloc((void**)&saveVel, sizeof(float4) * n));
    TUNE_CUDA(cudaMemcpyAsync(savePos, s->pos, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st));
    TUNE_CUDA(cudaMemcpyAsync(saveVel, s->vel, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st));
    const unsigned int steps0 = s->numTimeSteps;
    const bool stepped0 = s->stepped;
    float bestStep = 3.0e38f;
    StepConfig chosenCfg = current;
    cudaError_t te = cudaSuccess;
    for (const StepConfig& c : finalists) {
        s->cfg = c;
        invalidate_graphs(s);
        float fastest = 3.0e38f;
        for (int r = 0; r < 3 && te == cudaSuccess; r++) {
            te = cudaMemcpyAsync(s->pos, savePos, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
            if (te == cudaSuccess) te = cudaMemcpyAsync(s->vel, saveVel, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
            if (te == cudaSuccess && sph_step_many(s, SPH_STEP_PLAIN, 2) != SPH_OK) te = cudaErrorUnknown;  // capture
            if (te == cudaSuccess) te = cudaEventRecord(e0, st);
            if (te == cudaSuccess && sph_step_many(s, SPH_STEP_PLAIN, 8) != SPH_OK) te = cudaErrorUnknown;
            if (te == cudaSuccess) te = cudaEventRecord(e1, st);
            if (te == cudaSuccess) te = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
            if (te == cudaSuccess) fastest = std::min(fastest, ms);
        }
        // keep the incumbent unless beaten by 2 %
        if (te == cudaSuccess && fastest < (&c == &finalists[0] ? bestStep : 0.98f * bestStep)) {
            bestStep = fastest;
            chosenCfg = c;
        }
    }
    if (te == cudaSuccess) te = cudaMemcpyAsync(s->pos, savePos, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
    if (te == cudaSuccess) te = cudaMemcpyAsync(s->vel, saveVel, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st);
    if (te == cudaSuccess) te = cudaMemsetAsync(s->reuse, 0, sizeof(int), st);
    for (auto& b : bufs)
        if (te == cudaSuccess) te = cudaMemcpyAsync(b.dst, b.save, b.bytes, cudaMemcpyDeviceToDevice, st);
    if (te == cudaSuccess) te = cudaStreamSynchronize(st);
    cudaFree(savePos);
    cudaFree(saveVel);
    s->numTimeSteps = steps0;
    s->stepped = stepped0;
    TUNE_CUDA(te);
#undef TUNE_CUDA
    cleanup();
    s->cfg = chosenCfg;
    invalidate_graphs(s);
    if (chosen) return sph_get_tuning(s, chosen);
    return SPH_OK;
}

sph_status sph_time_kernel(sph_handle s, int stage, int reps, float* microseconds) {
    if (!s || !microseconds) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (stage != ST_DENSITY && stage != ST_FORCE)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "only the density and force stages repeat on one sorted state");
    if (reps < 1) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "reps must be positive");
    if (!s->stepped) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no step has run yet");
    cudaStream_t st = s->stream;
    const int n = s->n;
    GridDev g = grid_of(s);
    PhysDev ph = make_phys(s->P, s->O);
    // the density stage rewrites what it wrote (and the masks the force form
    // reads); the force stage rewrites the state the last step wrote
    SPH_CUDA(cudaMemsetAsync(s->reuse, 0, sizeof(int), st));
    // after a step over the reused neighbour lists the list forms are timed
    // (the density stage's list form: the lists match the sorted copies)
    const bool lists = s->vlOn && s->lastStepLists;
    if (lists)
        SPH_CUDA(cudaMemsetAsync(s->vl.flags + VL_BUILD_NOW * s->vl.numScenes, 0,
                                 sizeof(unsigned int) * s->vl.numScenes, st));
    auto launch = [&]() {
        if (lists) {
            if (stage == ST_DENSITY)
                launch_density_lists(n, s->posS, s->velS, rows_of(s), g, ph, s->map, s->rho4S, s->vl, s->cfg, false, true,
                                     st);
            else
                launch_force_lists(n, s->posS, s->velS, s->rho4S, s->sb.workIds, ph, s->map, s->O.boxCollision,
                                   s->vl, s->pos, s->vel, s->accS, s->cfg, st, s->sb.scenes);
        } else if (stage == ST_DENSITY) {
            launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, s->cfg, st);
        } else {
            launch_force(n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), g, ph, s->map,
                         s->O.boxCollision, s->rowStart, s->rowMask, s->pos, s->vel, s->accS, s->cfg, st, nullptr,
                         s->status);
        }
    };
    if (stage == ST_FORCE) {  // the masks of the current tuning
        StepConfig c = s->cfg;
        if (lists)
            launch_density_lists(n, s->posS, s->velS, rows_of(s), g, ph, s->map, s->rho4S, s->vl, c, false, true, st);
        else
            launch_density(n, s->posS, rows_of(s), g, ph, s->map, s->rho4S, s->rowStart, s->rowMask, c, st);
    }
    launch();  // warm
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SPH_CUDA(cudaEventCreate(&e0));
    cudaError_t e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) {
        for (int r = 0; r < reps; r++) launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    SPH_CUDA(e);
    *microseconds = 1e3f * ms / (float)reps;
    return latched_status(s);
}

sph_status sph_neighbour_builds(sph_handle s, unsigned int* builds) {
    if (!s || !builds) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    *builds = 0;
    if (!s->vlOn) return SPH_OK;
    // a batch: the scenes' builds summed
    std::vector<unsigned int> c((size_t)s->vl.numScenes);
    SPH_CUDA(cudaMemcpyAsync(c.data(), s->vl.flags + VL_COUNT * s->vl.numScenes, sizeof(unsigned int) * c.size(),
                             cudaMemcpyDeviceToHost, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    for (unsigned int v : c) *builds += v;
    return latched_status(s);
}

sph_status sph_stage_times(sph_handle s, float* ms, int* counts, int capacity, int* numStages) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (numStages) *numStages = ST_COUNT;
    if (!ms || capacity < ST_COUNT) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "capacity too small");
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < ST_COUNT; k++) {
        ms[k] = 0.0f;
        if (counts) counts[k] = 0;
    }
    for (int slot = 0; slot < s->timingFilled; slot++) {
        cudaEvent_t* ev = &s->events[(size_t)slot * (ST_COUNT + 1)];
        for (int k = 0; k < ST_COUNT; k++) {
            if (!(s->timingRan[slot] >> k & 1u)) continue;
            float t = 0.0f;
            SPH_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            ms[k] += t;
            if (counts) counts[k]++;
        }
    }
    s->timingNext = s->timingFilled = 0;
    return SPH_OK;
}

}  // extern "C"
