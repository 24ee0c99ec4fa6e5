// Host side of the learned step corrector: sample generation from the plain
// solver's trajectory, standardisation, Adam training, the learned step and
// its audit against the plain solver, and the checking entry points.
//
// Samples.  The handle runs trainSteps plain steps of dt.  For every start
// state S_k with S_{k+stride} known, a shadow handle runs one plain step of
// stride*dt from S_k; the sample is (features of S_k, S_{k+stride} minus the
// shadow's result).  The samples stay on the device.
//
// Learned step.  Hash, sort, density and force + integration with stride*dt,
// then the features of the pre-step state and the MLP, which adds its
// correction to positions and velocities (and collides again).
//
// Audit.  Every auditInterval-th learned step runs from a saved copy of the
// state both as a learned step and as `stride` plain steps of dt; densities
// of both results are computed (over the reused lists when the handle has
// them) and when the largest per-particle relative difference exceeds
// densityTolerance the plain result is kept.  The choice
// is made on the device, so learned and audit steps are each one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sph_corrector.h"
#include "sph_sim.h"

using namespace sph;
using namespace sph::mlp;

namespace sph {

struct Corrector {
    sph_corrector_config cfg{};
    bool ready = false;
    // model
    float *master = nullptr, *m1 = nullptr, *m2 = nullptr;
    unsigned char* image = nullptr;
    float* bias = nullptr;
    float* norm = nullptr;
    float stats[NSTATS] = {};  // feature means, deviations; target means, deviations, scales
    // learned step and audit scratch
    float* feat = nullptr;  // n x 24, particle order: the last recorded learned step's features
    bool record = false;    // learned steps write their features to `feat`
    bool recorded = false;  // `feat` holds a learned step's features
    float4 *lPos = nullptr, *lVel = nullptr;
    float *rhoA = nullptr, *rhoB = nullptr;
    unsigned int* errBits = nullptr;
    unsigned int* counters = nullptr;  // audits, rollbacks, last error bits, max error bits
    // gradient rows of the checking entry points
    float* partial = nullptr;
    int partialRows = 0;
    // captured graphs of a learned step and of an audited one
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    unsigned int gen[2] = {0, 0};
    bool valid[2] = {false, false};
    int sinceAudit = 0;
    sph_corrector_report rep{};
};

}  // namespace sph

namespace {

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// U[0, 1) with 24-bit resolution from (seed, stream, index).
double uniform01(unsigned int seed, uint64_t stream, uint64_t i) {
    const uint64_t z = splitmix64(((uint64_t)seed << 40) ^ (stream << 32) ^ i);
    return (double)(z >> 40) * (1.0 / (1 << 24));
}

MlpDev mdev(const Corrector* C) { return MlpDev{C->image, C->bias, C->norm}; }

PhysDev learned_phys(const sph_sim* s, int stride) {
    PhysDev ph = make_phys(s->P, s->O);
    ph.dt = (float)stride * s->P.timeStep;
    ph.dtCollide = ph.dt;
    return ph;
}

sph_status check_config(const sph_corrector_config* c) {
    if (!c) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "corrector config is NULL");
    if (c->stride < 1 || c->stride > 64) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "stride must be in [1, 64]");
    if (c->auditInterval < 0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "auditInterval must be >= 0");
    if (!(c->densityTolerance >= 0.0f)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "densityTolerance must be >= 0");
    if (!(c->targetScale >= 0.0f)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "targetScale must be >= 0");
    return SPH_OK;
}

void free_graphs(Corrector* C) {
    for (int k = 0; k < 2; k++) {
        if (C->exec[k]) cudaGraphExecDestroy(C->exec[k]);
        if (C->graph[k]) cudaGraphDestroy(C->graph[k]);
        C->exec[k] = nullptr;
        C->graph[k] = nullptr;
        C->valid[k] = false;
    }
}

sph_status ensure_corrector(sph_sim* s) {
    if (s->numScenes > 1) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "batched handles take plain steps only");
    if (s->corr) return SPH_OK;
    Corrector* C = new Corrector();
    s->corr = C;
    const size_t n = (size_t)s->n;
    SPH_CUDA(dalloc(&C->master, NPARAM));
    SPH_CUDA(dalloc(&C->m1, NPARAM));
    SPH_CUDA(dalloc(&C->m2, NPARAM));
    SPH_CUDA(dalloc(&C->image, IMG_BYTES));
    SPH_CUDA(dalloc(&C->bias, NBIAS));
    SPH_CUDA(dalloc(&C->norm, NNORM));
    SPH_CUDA(dalloc(&C->feat, n * IN));
    SPH_CUDA(dalloc(&C->lPos, n));
    SPH_CUDA(dalloc(&C->lVel, n));
    SPH_CUDA(dalloc(&C->rhoA, n));
    SPH_CUDA(dalloc(&C->rhoB, n));
    SPH_CUDA(dalloc(&C->errBits, 1));
    SPH_CUDA(dalloc(&C->counters, 4));
    SPH_CUDA(cudaMemsetAsync(C->image, 0, IMG_BYTES, s->stream));
    SPH_CUDA(cudaMemsetAsync(C->counters, 0, sizeof(unsigned int) * 4, s->stream));
    return SPH_OK;
}

sph_status ensure_partial(Corrector* C, int rows) {
    if (C->partialRows >= rows) return SPH_OK;
    if (C->partial) cudaFree(C->partial);
    C->partial = nullptr;
    C->partialRows = 0;
    SPH_CUDA(dalloc(&C->partial, (size_t)rows * PARTIAL));
    C->partialRows = rows;
    return SPH_OK;
}

// Standardisation of the device-side statistics (means and deviations).
void upload_norm(sph_sim* s, Corrector* C) {
    float h[NNORM] = {};
    for (int k = 0; k < IN; k++) {
        h[N_MUX + k] = C->stats[k];
        const float sd = C->stats[IN + k];
        h[N_ISX + k] = sd > 1e-8f ? 1.0f / sd : 0.0f;  // a constant feature carries nothing
    }
    for (int o = 0; o < OUT; o++) {
        h[N_MUT + o] = C->stats[2 * IN + o];
        const float sd = C->stats[2 * IN + OUT + o];
        h[N_SGT + o] = sd > 0.0f ? sd : 1.0f;
        h[N_SCL + o] = C->stats[2 * IN + 2 * OUT + o];
    }
    cudaMemcpyAsync(C->norm, h, sizeof(h), cudaMemcpyHostToDevice, s->stream);
}

// The learned step: a plain step of stride*dt, then features and correction.
// One learned step.  With reused neighbour lists on, its sort and density
// are those of a list step (the lists built when the decision says so, the
// distance a particle may move before a rebuild being the same for the long
// step) and the fused force stage walks the lists; otherwise the per-step
// search with its recorded masks.
void enqueue_learned(sph_sim* s, Corrector* C) {
    const int K = C->cfg.stride;
    const int n = s->n;
    cudaStream_t st = s->stream;
    GridDev g = grid_of(s);
    PhysDev ph = learned_phys(s, K);
    StepConfig cfg = s->cfg;
    const FeatureOut fo{C->record ? C->feat : nullptr, 1, s->O.boxCollision, ph.dt};
    if (s->vlOn) {
        launch_hash_count(n, s->pos, g, s->sb, s->status, st, &s->vl);
        launch_cell_scan(g.numCells, s->sb, s->status, st, &s->vl);
        launch_scatter(n, s->sb, st, s->status, &s->vl);
        launch_rank_gather(n, s->sb, s->pos, s->vel, g, s->posS, s->velS, st, &s->vl, s->status);
        launch_density_lists(n, s->posS, s->velS, rows_of(s), g, ph, s->map, s->rho4S, s->vl, cfg, true, true, st);
        // the sorted copies are now this step's own: a reuse the audit granted is used up
        cudaMemsetAsync(s->reuse, 0, sizeof(int), st);
        launch_force_learned(n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), g, ph, s->map,
                             s->O.boxCollision, nullptr, nullptr, s->pos, s->vel, s->accS, cfg, fo, mdev(C),
                             s->status, st, &s->vl);
        s->lastStepLists = true;
        return;
    }
    enqueue_coarse(s, g, ph, s->O.boxCollision, nullptr, nullptr, false);
    cfg.forceVariant = FORCE_PRETESTED;
    launch_force_learned(n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), g, ph, s->map,
                         s->O.boxCollision, s->rowStart, s->rowMask, s->pos, s->vel, s->accS, cfg, fo, mdev(C),
                         s->status, st);
}

void enqueue_audit(sph_sim* s, Corrector* C) {
    const size_t bytes = sizeof(float4) * (size_t)s->n;
    cudaStream_t q = s->stream;
    enqueue_learned(s, C);
    cudaMemcpyAsync(C->lPos, s->pos, bytes, cudaMemcpyDeviceToDevice, q);
    cudaMemcpyAsync(C->lVel, s->vel, bytes, cudaMemcpyDeviceToDevice, q);
    // The plain solver from the same start: its first step's sort and density
    // are the learned step's (neither depends on dt, and the sorted copies
    // still hold the start state), so only its force stage runs, over the
    // same neighbours; it writes every particle's new state.
    if (s->vlOn)
        launch_force_lists(s->n, s->posS, s->velS, s->rho4S, s->sb.workIds, make_phys(s->P, s->O), s->map,
                           s->O.boxCollision, s->vl, s->pos, s->vel, s->accS, s->cfg, q);
    else
        launch_force(s->n, s->posS, s->velS, s->rho4S, s->sb.workIds, rows_of(s), grid_of(s),
                     make_phys(s->P, s->O), s->map, s->O.boxCollision, s->rowStart, s->rowMask, s->pos, s->vel,
                     s->accS, s->cfg, q, nullptr, s->status);
    // the rest of the plain solver, as the first plain step above: over the
    // learned step's lists (reused while they hold) or with the per-step search
    for (int k = 1; k < C->cfg.stride; k++) enqueue_step(s, SPH_STEP_PLAIN, false, s->vlOn);
    if (s->vlOn) {
        // Both densities over the lists, as a list step takes its density:
        // the plain result's (its distance from the build positions is the
        // one its last force stage recorded), then the learned result's
        // after measuring its own distance (a build it needs centres the
        // lists on it).  Then the kept state's distance, for the next step.
        enqueue_list_density(s, s->pos, s->vel);
        launch_unpermute(s->n, s->sb.workIds, s->rho4S, 0, C->rhoB, 1, 0, q);
        launch_list_displacement(s->n, C->lPos, s->sb.workIds, s->vl, q);
        enqueue_list_density(s, C->lPos, C->lVel);
        launch_unpermute(s->n, s->sb.workIds, s->rho4S, 0, C->rhoA, 1, 0, q);
        cudaMemsetAsync(C->errBits, 0, sizeof(unsigned int), q);
        launch_audit(s->n, C->rhoA, C->rhoB, C->errBits, q);
        launch_audit_select(s->n, C->errBits, C->cfg.densityTolerance, C->lPos, C->lVel, s->pos, s->vel,
                            C->counters, nullptr, q);
        launch_list_displacement(s->n, s->pos, s->sb.workIds, s->vl, q);
        return;
    }
    enqueue_density_only(s, s->pos, s->vel);
    launch_unpermute(s->n, s->sb.workIds, s->rho4S, 0, C->rhoB, 1, 0, q);
    // last: the learned result, with the neighbour masks, so that when the
    // audit keeps it the next step finds its sort and density done
    enqueue_density_only(s, C->lPos, C->lVel, true);
    launch_unpermute(s->n, s->sb.workIds, s->rho4S, 0, C->rhoA, 1, 0, q);
    cudaMemsetAsync(C->errBits, 0, sizeof(unsigned int), q);
    launch_audit(s->n, C->rhoA, C->rhoB, C->errBits, q);
    launch_audit_select(s->n, C->errBits, C->cfg.densityTolerance, C->lPos, C->lVel, s->pos, s->vel, C->counters,
                        s->reuse, q);
}

void enqueue_kind(sph_sim* s, Corrector* C, int kind) {
    if (kind == 0) enqueue_learned(s, C);
    else enqueue_audit(s, C);
}

sph_status launch_kind(sph_sim* s, Corrector* C, int kind) {
    if (s->timingCap > 0) {
        enqueue_kind(s, C, kind);
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }
    if (!C->valid[kind] || C->gen[kind] != s->graphGen) {
        if (C->exec[kind]) cudaGraphExecDestroy(C->exec[kind]);
        if (C->graph[kind]) cudaGraphDestroy(C->graph[kind]);
        C->exec[kind] = nullptr;
        C->graph[kind] = nullptr;
        SPH_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_kind(s, C, kind);
        cudaGraph_t g = nullptr;
        SPH_CUDA(cudaStreamEndCapture(s->stream, &g));
        C->graph[kind] = g;
        SPH_CUDA(cudaGraphInstantiate(&C->exec[kind], g, 0));
        C->valid[kind] = true;
        C->gen[kind] = s->graphGen;
    }
    SPH_CUDA(cudaGraphLaunch(C->exec[kind], s->stream));
    return SPH_OK;
}

}  // namespace

namespace sph {

void corrector_free(sph_sim* s) {
    Corrector* C = s->corr;
    if (!C) return;
    free_graphs(C);
    void* ptrs[] = {C->master, C->m1,   C->m2,   C->image,  C->bias,     C->norm,    C->feat,
                    C->lPos, C->lVel, C->rhoA, C->rhoB, C->errBits,
                    C->counters, C->partial};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete C;
    s->corr = nullptr;
}

sph_status corrector_step(sph_sim* s, int count, bool useGraph) {
    Corrector* C = s->corr;
    if (!C || !C->ready)
        SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "SPH_STEP_LEARNED needs a trained or loaded corrector");
    for (int i = 0; i < count; i++) {
        const bool audit = C->cfg.auditInterval > 0 && C->sinceAudit + 1 >= C->cfg.auditInterval;
        const int kind = audit ? 1 : 0;
        if (useGraph) {
            sph_status st = launch_kind(s, C, kind);
            if (st) return st;
        } else {
            enqueue_kind(s, C, kind);
            SPH_CUDA(cudaGetLastError());
        }
        C->sinceAudit = audit ? 0 : C->sinceAudit + 1;
        // learned steps and audits over the lists leave sorted copies that
        // match the lists (an audit: the learned result's, and the kept
        // state's distance from the build positions recorded)
        s->lastStepLists = s->vlOn;
        C->rep.learnedSteps++;
        C->recorded = C->recorded || C->record;
    }
    s->numTimeSteps += (unsigned int)count;
    s->stepped = true;
    return SPH_OK;
}

}  // namespace sph

extern "C" {

void sph_corrector_default_config(sph_corrector_config* c) {
    if (!c) return;
    c->trainSteps = 2000;
    c->stride = 4;
    c->epochs = 6;
    c->batchTiles = 128;
    c->learningRate = 2e-3f;
    c->densityTolerance = 0.01f;
    c->auditInterval = 16;
    c->seed = 1;
    c->targetScale = 0.0f;
}

sph_status sph_corrector_train(sph_handle s, const sph_corrector_config* cfg) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    sph_status st = check_config(cfg);
    if (st) return st;
    if (cfg->trainSteps < cfg->stride) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "trainSteps must be >= stride");
    if (s->O.cellRelative) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "the corrector takes absolute positions");
    if (cfg->epochs < 1 || cfg->batchTiles < 1) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "epochs and batchTiles >= 1");
    if (!(cfg->learningRate > 0.0f)) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "learningRate must be positive");
    st = ensure_corrector(s);
    if (st) return st;
    Corrector* C = s->corr;
    C->cfg = *cfg;
    C->ready = false;
    free_graphs(C);
    cudaStream_t q = s->stream;
    const int n = s->n;
    const int K = cfg->stride;
    const long long sets = (long long)cfg->trainSteps - K + 1;
    const long long rows = sets * n;
    if (rows > (long long)INT32_MAX * TILE) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "too many training samples");

    // sample buffers, the ring of the last stride+1 states, the shadow handle
    float *feat = nullptr, *tgt = nullptr;
    float4* ring = nullptr;
    double *statP = nullptr, *statOut = nullptr;
    float* lossBuf = nullptr;
    int* tileList = nullptr;
    sph_handle sh = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        if (sh) sph_destroy(sh);
        void* ptrs[] = {feat, tgt, ring, statP, statOut, lossBuf, tileList};
        for (void* p : ptrs)
            if (p) cudaFree(p);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
#define TRAIN_CUDA(call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            cleanup();                                                                                \
            return record_error(e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA, \
                                __FILE__, __LINE__, cudaGetErrorString(e_));                          \
        }                                                                                             \
    } while (0)
#define TRAIN_ST(expr)          \
    do {                        \
        sph_status s_ = (expr); \
        if (s_) {               \
            cleanup();          \
            return s_;          \
        }                       \
    } while (0)
    TRAIN_CUDA(dalloc(&feat, (size_t)rows * IN));
    TRAIN_CUDA(dalloc(&tgt, (size_t)rows * TGT));
    TRAIN_CUDA(dalloc(&ring, (size_t)2 * (K + 1) * n));
    TRAIN_CUDA(dalloc(&statP, (size_t)304 * 48));
    TRAIN_CUDA(dalloc(&statOut, 64));
    TRAIN_CUDA(cudaEventCreate(&e0));
    TRAIN_CUDA(cudaEventCreate(&e1));
    {
        std::vector<float> host((size_t)n * 3);
        TRAIN_ST(sph_read(s, SPH_FIELD_VERTEX_DATA, host.data(), host.size() * sizeof(float)));
        TRAIN_ST(sph_create(&s->P, &s->O, host.data(), nullptr, nullptr, &sh));
    }
    sh->map = s->map;  // the shadow reads the handle's boundary maps (it owns none)
    TRAIN_ST(sph_set_stream(sh, q));
    sh->cfg = s->cfg;
    TRAIN_CUDA(cudaEventRecord(e0, q));
    const GridDev g = grid_of(s);
    const PhysDev ph4 = learned_phys(s, K);
    const size_t bytes = sizeof(float4) * (size_t)n;
    for (int i = 0; i <= cfg->trainSteps; i++) {
        float4* slot = ring + (size_t)2 * (i % (K + 1)) * n;
        TRAIN_CUDA(cudaMemcpyAsync(slot, s->pos, bytes, cudaMemcpyDeviceToDevice, q));
        TRAIN_CUDA(cudaMemcpyAsync(slot + n, s->vel, bytes, cudaMemcpyDeviceToDevice, q));
        if (i >= K) {
            const long long k = i - K;
            const float4* start = ring + (size_t)2 * (k % (K + 1)) * n;
            TRAIN_CUDA(cudaMemcpyAsync(sh->pos, start, bytes, cudaMemcpyDeviceToDevice, q));
            TRAIN_CUDA(cudaMemcpyAsync(sh->vel, start + n, bytes, cudaMemcpyDeviceToDevice, q));
            const FeatureOut fo{feat + (size_t)k * n * IN, 1, s->O.boxCollision, ph4.dt};
            enqueue_coarse(sh, g, ph4, s->O.boxCollision, nullptr, &fo);
            launch_targets(n, s->pos, s->vel, sh->pos, sh->vel, tgt + (size_t)k * n * TGT, q);
        }
        if (i < cfg->trainSteps) TRAIN_ST(sph_step_many(s, SPH_STEP_PLAIN, 1));
    }
    TRAIN_CUDA(cudaGetLastError());
    TRAIN_ST(latched_status(sh));
    TRAIN_ST(latched_status(s));
    sph_destroy(sh);
    sh = nullptr;

    // standardisation
    {
        double h[64];
        launch_column_stats(rows, IN, IN, feat, statP, statOut, q);
        TRAIN_CUDA(cudaMemcpyAsync(h, statOut, sizeof(double) * 2 * IN, cudaMemcpyDeviceToHost, q));
        TRAIN_CUDA(cudaStreamSynchronize(q));
        for (int k = 0; k < IN; k++) {
            C->stats[k] = (float)h[2 * k];
            C->stats[IN + k] = (float)h[2 * k + 1];
        }
        // targets: with targetScale > 0 the network predicts asinh(t/s), s a
        // fraction of each component's deviation (s = 0: t itself)
        launch_column_stats(rows, OUT, TGT, tgt, statP, statOut, q);
        TRAIN_CUDA(cudaMemcpyAsync(h, statOut, sizeof(double) * 2 * OUT, cudaMemcpyDeviceToHost, q));
        TRAIN_CUDA(cudaStreamSynchronize(q));
        TargetScales sc{};
        for (int o = 0; o < OUT; o++) sc.s[o] = (float)((double)cfg->targetScale * h[2 * o + 1]);
        float* ttmp = nullptr;
        TRAIN_CUDA(dalloc(&ttmp, (size_t)rows * TGT));
        launch_target_transform(rows, tgt, sc, ttmp, q);
        launch_column_stats(rows, OUT, TGT, ttmp, statP, statOut, q);
        cudaError_t e = cudaMemcpyAsync(h, statOut, sizeof(double) * 2 * OUT, cudaMemcpyDeviceToHost, q);
        if (e == cudaSuccess) e = cudaStreamSynchronize(q);
        cudaFree(ttmp);
        TRAIN_CUDA(e);
        for (int o = 0; o < OUT; o++) {
            C->stats[2 * IN + o] = (float)h[2 * o];
            C->stats[2 * IN + OUT + o] = (float)h[2 * o + 1];
            C->stats[2 * IN + 2 * OUT + o] = sc.s[o];
        }
        upload_norm(s, C);
    }

    // initial weights: uniform(+-1/sqrt(fan in)), the last layer 10x smaller
    {
        std::vector<float> w(NPARAM, 0.0f);
        for (int o = 0; o < HID; o++)
            for (int i = 0; i < IN; i++)
                w[P_W1 + o * INP + i] = (float)((2.0 * uniform01(cfg->seed, 1, o * INP + i) - 1.0) / std::sqrt(24.0));
        for (int o = 0; o < HID; o++)
            for (int i = 0; i < HID; i++)
                w[P_W2 + o * HID + i] = (float)((2.0 * uniform01(cfg->seed, 2, o * HID + i) - 1.0) / 8.0);
        for (int o = 0; o < OUT; o++)
            for (int i = 0; i < HID; i++)
                w[P_W3 + o * HID + i] = (float)((2.0 * uniform01(cfg->seed, 3, o * HID + i) - 1.0) / 80.0);
        TRAIN_CUDA(cudaMemcpyAsync(C->master, w.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, q));
        TRAIN_CUDA(cudaMemsetAsync(C->m1, 0, sizeof(float) * NPARAM, q));
        TRAIN_CUDA(cudaMemsetAsync(C->m2, 0, sizeof(float) * NPARAM, q));
        launch_mlp_pack(C->master, C->image, C->bias, q);
        TRAIN_CUDA(cudaStreamSynchronize(q));  // `w` leaves scope
    }

    // Adam over shuffled 128-sample tiles
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (rows + TILE - 1) / TILE;
    const int batch = (int)std::min<long long>(cfg->batchTiles, tiles);
    int ctas = std::min(batch, sms);
    while (batch % ctas) ctas--;
    const int perCta = batch / ctas;
    const long long stepsPerEpoch = tiles / batch;
    const long long total = stepsPerEpoch * cfg->epochs;
    TRAIN_ST(ensure_partial(C, ctas));
    TRAIN_CUDA(dalloc(&lossBuf, (size_t)total));
    TRAIN_CUDA(dalloc(&tileList, (size_t)tiles));
    std::vector<int> order((size_t)tiles);
    const float invScale = 1.0f / (6.0f * (float)batch * (float)TILE);
    long long u = 0;
    for (int ep = 0; ep < cfg->epochs; ep++) {
        for (long long t = 0; t < tiles; t++) order[(size_t)t] = (int)t;
        for (long long t = tiles - 1; t > 0; t--) {  // Fisher-Yates
            const uint64_t r = splitmix64(((uint64_t)cfg->seed << 40) ^ ((uint64_t)(ep + 16) << 32) ^ (uint64_t)t);
            const long long j = (long long)(r % (uint64_t)(t + 1));
            std::swap(order[(size_t)t], order[(size_t)j]);
        }
        TRAIN_CUDA(cudaMemcpyAsync(tileList, order.data(), sizeof(int) * (size_t)tiles, cudaMemcpyHostToDevice, q));
        for (long long b = 0; b < stepsPerEpoch; b++, u++) {
            const float lr = cfg->learningRate * (1.0f - 0.99f * (float)u / (float)std::max<long long>(total, 1));
            launch_mlp_grad(ctas, perCta, tileList + b * batch, feat, tgt, rows, invScale, mdev(C), C->partial,
                            s->status, q);
            launch_mlp_adam(ctas, C->partial, C->master, C->m1, C->m2, (int)std::min<long long>(u + 1, 1 << 30), lr, 1,
                            C->image, C->bias, nullptr, lossBuf + u, q);
        }
        TRAIN_CUDA(cudaStreamSynchronize(q));  // `order` is rewritten next epoch
    }
    TRAIN_CUDA(cudaEventRecord(e1, q));
    TRAIN_CUDA(cudaGetLastError());
    TRAIN_ST(latched_status(s));
    std::vector<float> losses((size_t)total);
    if (total > 0)
        TRAIN_CUDA(cudaMemcpy(losses.data(), lossBuf, sizeof(float) * (size_t)total, cudaMemcpyDeviceToHost));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    auto epochMean = [&](int ep) {
        double sum = 0.0;
        for (long long b = 0; b < stepsPerEpoch; b++) sum += losses[(size_t)(ep * stepsPerEpoch + b)];
        return (float)(sum / ((double)std::max<long long>(stepsPerEpoch, 1) * 6.0 * batch * TILE));
    };
    C->rep.samples = (unsigned int)std::min<long long>(rows, 0xFFFFFFFFll);
    C->rep.optimizerSteps = (unsigned int)total;
    C->rep.firstEpochLoss = stepsPerEpoch > 0 ? epochMean(0) : 0.0f;
    C->rep.lastEpochLoss = stepsPerEpoch > 0 ? epochMean(cfg->epochs - 1) : 0.0f;
    C->rep.trainMilliseconds = ms;
    C->ready = true;
    C->sinceAudit = 0;
    cleanup();
#undef TRAIN_CUDA
#undef TRAIN_ST
    return SPH_OK;
}

sph_status sph_corrector_load(sph_handle s, const sph_corrector_config* cfg, const float* model, size_t count) {
    if (!s || !model) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    sph_status st = check_config(cfg);
    if (st) return st;
    if (count < (size_t)SPH_CORRECTOR_FLOATS) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "model blob too small");
    if (s->O.cellRelative) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "the corrector takes absolute positions");
    st = ensure_corrector(s);
    if (st) return st;
    Corrector* C = s->corr;
    C->cfg = *cfg;
    free_graphs(C);
    SPH_CUDA(cudaMemcpyAsync(C->master, model, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, s->stream));
    SPH_CUDA(cudaMemsetAsync(C->m1, 0, sizeof(float) * NPARAM, s->stream));
    SPH_CUDA(cudaMemsetAsync(C->m2, 0, sizeof(float) * NPARAM, s->stream));
    std::memcpy(C->stats, model + NPARAM, sizeof(C->stats));
    upload_norm(s, C);
    launch_mlp_pack(C->master, C->image, C->bias, s->stream);
    SPH_CUDA(cudaGetLastError());
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    C->ready = true;
    C->sinceAudit = 0;
    return SPH_OK;
}

sph_status sph_corrector_save(sph_handle s, float* model, size_t count) {
    if (!s || !model) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->corr || !s->corr->ready) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "no trained or loaded corrector");
    if (count < (size_t)SPH_CORRECTOR_FLOATS) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "model buffer too small");
    SPH_CUDA(cudaMemcpyAsync(model, s->corr->master, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s->stream));
    SPH_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(model + NPARAM, s->corr->stats, sizeof(s->corr->stats));
    return SPH_OK;
}

sph_status sph_corrector_get_report(sph_handle s, sph_corrector_report* out) {
    if (!s || !out) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    if (!s->corr) return SPH_OK;
    Corrector* C = s->corr;
    unsigned int c[4];
    SPH_CUDA(cudaMemcpyAsync(c, C->counters, sizeof(c), cudaMemcpyDeviceToHost, s->stream));
    sph_status st = latched_status(s);
    if (st) return st;
    *out = C->rep;
    out->audits = c[0];
    out->rollbacks = c[1];
    std::memcpy(&out->lastAuditError, &c[2], sizeof(float));
    std::memcpy(&out->maxAuditError, &c[3], sizeof(float));
    return SPH_OK;
}

sph_status sph_corrector_predict(sph_handle s, const float* features, int count, float* corrections) {
    if (!s || !features || !corrections) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->corr || !s->corr->ready) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "no trained or loaded corrector");
    if (count <= 0) return SPH_OK;
    Corrector* C = s->corr;
    float *f = nullptr, *o = nullptr;
    SPH_CUDA(dalloc(&f, (size_t)count * IN));
    if (dalloc(&o, (size_t)count * OUT) != cudaSuccess) {
        cudaFree(f);
        SPH_FAIL(SPH_ERR_OUT_OF_MEMORY, "corrector output");
    }
    cudaStream_t q = s->stream;
    cudaMemcpyAsync(f, features, sizeof(float) * (size_t)count * IN, cudaMemcpyHostToDevice, q);
    launch_mlp_apply(count, f, mdev(C), 1, nullptr, nullptr, nullptr, make_phys(s->P, s->O), 0, o, s->status, q);
    cudaError_t e = cudaMemcpyAsync(corrections, o, sizeof(float) * (size_t)count * OUT, cudaMemcpyDeviceToHost, q);
    cudaStreamSynchronize(q);
    cudaFree(f);
    cudaFree(o);
    SPH_CUDA(e);
    SPH_CUDA(cudaGetLastError());
    return latched_status(s);
}

sph_status sph_corrector_gradient(sph_handle s, const float* features, const float* targets, int count, float* grad,
                                  float* loss) {
    if (!s || !features || !targets || !grad || !loss) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->corr || !s->corr->ready) SPH_FAIL(SPH_ERR_NOT_SUPPORTED, "no trained or loaded corrector");
    if (count <= 0) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "count must be positive");
    Corrector* C = s->corr;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (count + TILE - 1) / TILE;
    const int ctas = std::min(tiles, sms);
    const int perCta = (tiles + ctas - 1) / ctas;
    sph_status st = ensure_partial(C, ctas);
    if (st) return st;
    std::vector<int> list((size_t)ctas * perCta);
    for (size_t i = 0; i < list.size(); i++) list[i] = (int)std::min<size_t>(i, (size_t)tiles);
    float *f = nullptr, *t = nullptr, *gd = nullptr;
    int* l = nullptr;
    cudaStream_t q = s->stream;
    cudaError_t e = dalloc(&f, (size_t)count * IN);
    if (e == cudaSuccess) e = dalloc(&t, (size_t)count * TGT);
    if (e == cudaSuccess) e = dalloc(&gd, (size_t)NPARAM + 1);
    if (e == cudaSuccess) e = dalloc(&l, list.size());
    if (e == cudaSuccess) e = cudaMemcpyAsync(f, features, sizeof(float) * (size_t)count * IN, cudaMemcpyHostToDevice, q);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t, targets, sizeof(float) * (size_t)count * TGT, cudaMemcpyHostToDevice, q);
    if (e == cudaSuccess) e = cudaMemcpyAsync(l, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, q);
    if (e == cudaSuccess) {
        launch_mlp_grad(ctas, perCta, l, f, t, count, 1.0f / (6.0f * (float)count), mdev(C), C->partial, s->status, q);
        launch_mlp_adam(ctas, C->partial, C->master, C->m1, C->m2, 0, 0.0f, 0, C->image, C->bias, gd, gd + NPARAM, q);
        e = cudaMemcpyAsync(grad, gd, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, q);
        if (e == cudaSuccess) e = cudaMemcpyAsync(loss, gd + NPARAM, sizeof(float), cudaMemcpyDeviceToHost, q);
    }
    cudaStreamSynchronize(q);
    void* ptrs[] = {f, t, gd, l};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    SPH_CUDA(e);
    SPH_CUDA(cudaGetLastError());
    return latched_status(s);
}

sph_status sph_corrector_record_features(sph_handle s, int enable) {
    if (!s) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "handle is NULL");
    if (!s->corr || !s->corr->ready) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no corrector is loaded");
    Corrector* C = s->corr;
    if (C->record != (enable != 0)) {
        C->record = enable != 0;
        C->valid[0] = C->valid[1] = false;  // the captured steps change
    }
    return SPH_OK;
}

sph_status sph_read_features(sph_handle s, float* dst, size_t bytes) {
    if (!s || !dst) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->corr || !s->corr->recorded)
        SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "no learned step has run with feature recording on");
    const size_t need = sizeof(float) * (size_t)s->n * IN;
    if (bytes < need) SPH_FAIL(SPH_ERR_INVALID_ARGUMENT, "destination too small");
    SPH_CUDA(cudaMemcpyAsync(dst, s->corr->feat, need, cudaMemcpyDeviceToHost, s->stream));
    return latched_status(s);
}

}  // extern "C"
