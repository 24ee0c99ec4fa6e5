// The simulation handle behind the C ABI and the host helpers that the
// translation units orchestrating a step share (sph_api.cu, sph_corrector.cu).
// Not part of the public ABI.
#pragma once

#include <string>
#include <vector>

#include "sph_internal.h"

namespace sph {
// Records a failure in the per-thread message sph_last_error() returns and
// passes the status through (the reference's message shape, util.h:24-39).
sph_status record_error(sph_status st, const char* file, int line, const std::string& msg);
}  // namespace sph

#define SPH_FAIL(st, msg) return sph::record_error((st), __FILE__, __LINE__, (msg))
#define SPH_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            sph_status st_ = e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY      \
                                                             : SPH_ERR_CUDA;              \
            return sph::record_error(st_, __FILE__, __LINE__, cudaGetErrorString(e_));    \
        }                                                                                \
    } while (0)

namespace sph {

// The stages a step records events between (sph_set_stage_timing).  A plain
// step runs the first six; a two-scale step also the coarse-to-fine hand-over
// (states, split lists, children, projection) and the fine level's sort,
// density and force.
enum Stage {
    ST_HASH,
    ST_SCAN,
    ST_SCATTER,
    ST_RANK,
    ST_DENSITY,
    ST_FORCE,
    ST_TS_CHILDREN,
    ST_SUB_SORT,
    ST_SUB_DENSITY,
    ST_SUB_FORCE,
    ST_COUNT
};

template <class T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc((void**)p, sizeof(T) * (count > 0 ? count : 1));
}

struct Corrector;  // sph_corrector.cu

}  // namespace sph

struct sph_sim {
    SimulationParameters P;
    sph_options O;
    int n = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t ownStream = nullptr;

    // state (particle order) and per-step sorted copies
    float4 *pos = nullptr, *vel = nullptr;
    float4 *posS = nullptr, *velS = nullptr, *rho4S = nullptr, *accS = nullptr;
    int* rowStart = nullptr;          // [9][n] neighbour-row windows recorded by the density stage
    unsigned int* rowMask = nullptr;  // [9][n] their neighbour masks
    sph::SortBuffers sb{};
    unsigned long long* scanBlock = nullptr;
    unsigned int* status = nullptr;     // device status word
    int* reuse = nullptr;               // device flag: the sorted copies hold the current state
                                        // (set by an accepting audit, used up by the next step)
    unsigned int* statusHost = nullptr; // pinned copy
    float* staging = nullptr;           // device AoS staging, n*10 floats
    // Uploads from page-locked sources while the handle's stream is busy: DMA
    // copies on a stream of their own into landing buffers (AoS), unpacked on
    // the handle's stream once landed, so the host link and the work queued
    // there overlap.  Asynchronous reads: packed on the handle's stream into
    // a buffer of their own, copied to the host by DMA on another stream.
    cudaStream_t upStream = nullptr;
    float* upLand[2] = {nullptr, nullptr};           // positions, velocities: float[3n]
    cudaEvent_t upReady[2] = {nullptr, nullptr};     // landed
    cudaEvent_t upFree[2] = {nullptr, nullptr};      // unpacked: the landing buffer may be refilled
    cudaStream_t downStream = nullptr;
    float* downStage = nullptr;                      // float[3n]
    cudaEvent_t downReady = nullptr;                 // packed
    cudaEvent_t downFree = nullptr;                  // copied to the host: the buffer may be refilled
    std::vector<float> sdMass, sdEnergy;  // SD_MASS / SD_ENERGY columns (never touched by the step)

    // boundary maps
    float4* map4 = nullptr;
    float* mapDist = nullptr;
    sph::MapDev map{};

    unsigned int numTimeSteps = 0;
    bool stepped = false;

    // launch configuration
    sph::StepConfig cfg;

    // two-scale pass (allocated on first use)
    sph::TwoScaleDev ts{};
    sph::SortBuffers subSb{};
    unsigned long long* subScanBlock = nullptr;
    bool tsReady = false;

    // CUDA graph of one step of graphMode
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    bool graphValid = false;
    int graphMode = -1;
    unsigned int graphGen = 0;  // bumped whenever captured graphs go stale


    // cells owned by the handle: the grid's, or the sum over batched scenes
    long long numCellsTotal = 0;
    // batched scenes (sph_create_batch): count, first particle and first cell
    // of each scene (numScenes + 1 entries) and the device scene table
    int numScenes = 1;
    std::vector<unsigned int> sceneStart, sceneCell;
    sph::SceneDev* scenesDev = nullptr;

    // learned step corrector (sph_corrector.cu; allocated on first use)
    sph::Corrector* corr = nullptr;

    // FP64 diagnostics scratch: partial rows then the DIAG_TERMS results
    double* diagBuf = nullptr;

    // reused neighbour lists (sph_options.neighbourSkin > 0 on a single-scene
    // handle with absolute positions): plain steps build and reuse them
    sph::NeighbourLists vl{};
    bool vlOn = false;
    bool lastStepLists = false;  // the last step ran over the lists (they match the sorted copies)

    // stage timing ring
    int timingCap = 0, timingNext = 0, timingFilled = 0;
    std::vector<cudaEvent_t> events;  // timingCap * (sph::ST_COUNT + 1)
    std::vector<unsigned int> timingRan;  // per timed step: bit k set when stage k ran
};


namespace sph {

RowTables rows_of(const sph_sim* s);
GridDev make_grid(const SimulationParameters& P, bool sub);
PhysDev make_phys(const SimulationParameters& P, const sph_options& O);
PhysDev make_sub_phys(const SimulationParameters& P, const sph_options& O);
sph_status validate_params(const SimulationParameters* P, const sph_options* O);
sph_status check_desc(const sph_boundary_desc* d, unsigned int dims[3]);
void free_all(sph_sim* s);
sph_status ensure_two_scale(sph_sim* s);
// Enqueues one step of `mode` (no host synchronisation).  A plain step runs
// over the reused neighbour lists when the handle has them and `lists`.
void enqueue_step(sph_sim* s, int mode, bool timing, bool lists = true);
// Asks the next plain step over the lists to build them (the sorted copies
// and the working order changed under them).
void request_list_build(sph_sim* s);
// Allocates the reused neighbour lists when the handle's options ask for them.
sph_status alloc_lists(sph_sim* s);
// Radius and displacement limit of the lists from the handle's parameters.
void set_list_radius(sph_sim* s);
// Hash, sort, density and force + integration (+ box collision) of the
// coarse particles with the given constants; stage events when `ev`; the
// force stage also records the corrector's features when `feat`.  With
// `force` false it stops after the density stage (which then records the
// pretested neighbour masks), for a caller that runs its own force stage.
void enqueue_coarse(sph_sim* s, const GridDev& g, const PhysDev& ph, int collide, cudaEvent_t* ev,
                    const FeatureOut* feat = nullptr, bool force = true);
// Hash, sort and density of the state (pos, vel) into the handle's sorted
// copies (posS, velS, rho4S) and cell tables, with the neighbour masks when
// `masks`; nothing is integrated.
void enqueue_density_only(sph_sim* s, const float4* pos, const float4* vel, bool masks = false);
// The front of a step over the reused lists for the state (pos, vel): the
// decision (from the distance recorded for the lists), the sort stages when
// it builds, the gather into the working order and the density stage in the
// form the decision selects; nothing is integrated.
void enqueue_list_density(sph_sim* s, const float4* pos, const float4* vel);
// Marks every captured step graph of the handle stale.
void invalidate_graphs(sph_sim* s);

// The learned step corrector (sph_corrector.cu).
sph_status corrector_step(sph_sim* s, int count, bool useGraph);
void corrector_free(sph_sim* s);
// Waits for the handle's stream and maps the latched device status.
sph_status latched_status(sph_sim* s);
// The status held in statusHost (already copied back and synchronised).
sph_status status_of_host_copy(const sph_sim* s);
// Device address of page-locked host memory, or NULL (pageable memory).
void* host_device_ptr(const void* p);
// Allocates the device state of n particles over C cells (zeroed counters,
// velocities and per-step outputs) and the handle's stream.
sph_status alloc_handle(sph_sim* s, int n, long long C);
// Texture metadata of boundary maps built from `d` on a dims^3 grid.
MapDev map_of(const sph_boundary_desc& d, const unsigned int dims[3], const float4* map4, const float* dist);
// The coarse grid of the handle with numCells = all cells it owns (the sum
// over the scenes of a batched handle).
GridDev grid_of(const sph_sim* s);

}  // namespace sph
