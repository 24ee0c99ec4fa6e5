// Internal declarations shared by the kernels (sph_kernels.cu) and the host
// orchestration (sph_api.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sph.h"

namespace sph {

// Device-side status bits, latched per handle and mapped to sph_status.
enum : unsigned int {
    STATUS_OUT_OF_DOMAIN = 1u,
    STATUS_DEVICE_WAIT = 2u,
    STATUS_NON_FINITE = 4u,
};

// Uniform cell grid (gridOrigin/gridSpacing/gridDim of SimulationParameters).
struct GridDev {
    float origin[3];
    float spacing;
    int dim[3];
    int numCells;
    int cellBase;  // first global cell index of this grid (batched scenes; else 0)
    int rel;       // positions are cell-relative (sph_options.cellRelative)
};

// Largest grid of a cell-relative handle: cell coordinates pack 11:11:10 bits.
constexpr int REL_MAX_X = 2048, REL_MAX_Y = 2048, REL_MAX_Z = 1024;

// Trilinear boundary maps: map4 = (signed distance, wall density, wall
// viscosity, 0) per node, dist = signed distance alone (gradient samples).
struct MapDev {
    const float4* map4;
    const float* dist;
    float origin[3];
    float length[3];   // (dims-1)*spacing, particle_simulation.cu:2628-2631
    float dimsf[3];
    int dims[3];
    float du[3];       // spacing/length: the gradient step, :429-431
    float restDistance;
    int present;
};

// Per-level physical constants, pre-combined.
struct PhysDev {
    float h, h2;
    float poly6m;      // poly6 * mass
    float mass;
    float stiffness, restDensity;
    float pressCoef;   // -mass * gradSpiky (times rho_i per particle)
    float viscCoef;    // mu * mass * laplVisc
    float cgCoef;      // mass * gradPoly6
    float clCoef;      // mass * laplPoly6
    float tension, normThresh;
    float dt;          // integration step of this level
    float dtCollide;   // gSimParamsDev.timeStep (collision restitution term)
    float gravity;
    int gravityAxis;
    float boxCen[3], boxDim[3], restitution;
};

// One scene of a batched handle: its own cell grid (at cellBase in the
// concatenated cell space), physical constants, walls and boundary maps.  A
// particle's scene index travels in the .w lane of its position.
struct SceneDev {
    GridDev g;
    PhysDev ph;
    MapDev map;
};

// Scratch of the counting sort + cell scan.
struct SortBuffers {
    int* cnt;                 // [C+1] per-cell counters (kept zero between steps)
    int* cellOffset;          // [C+1] exclusive scan of cnt: first sorted index of each cell
    int2* keySlot;            // [n]   (hash, arrival slot in its cell)
    int* tmpIds;              // [n]   ids scattered to their cell segment, unordered
    int* sortedHash;          // [n]
    int* sortedIds;           // [n]   the reference's permutation (cell, id)
    int* workIds;             // [n]   the working order (cell, x, id) of the sorted arrays
    int* halfOffset;          // [C+1] first working index of each cell's upper x-half
                              //       (meaningful for occupied cells only)
    unsigned long long* scanFlags;  // decoupled look-back tile states
    unsigned int* tileCounter;
    int maxTiles;
    const SceneDev* scenes;   // batched handles: per-scene grids (else NULL)
    const int* skip;          // when non-NULL and set on the device, the sorted copies and
                              // tables already hold the current state: the sort stages return
};

// Two-scale state (AdvanceTwoScale): particle states, the three-way lists,
// persistent child slots 8*parent + k, and the fine level's sort.
struct TwoScaleDev {
    unsigned char* state;       // [n rounded up to 4] 2-bit history per particle
    int* blockCounts;           // [3 * blocks] per-block class counts
    int* counts;                // [5] split, boundary, default, children (device side); [4]: length
                                //     of markList, zero between steps
    int* markList;              // [n] working-order indices of split particles, any order
    int* splitIds;              // [n]
    int* boundaryIds;           // [n]
    int* defaultIds;            // [n]
    int* subIds;                // [8n] child list: split children, then boundary children
    float4* subPos;             // [8n] slots
    float4* subVel;
    float4* subAcc;
    float2* subRho;             // (density, pressure)
    int* subCnt;                // [Cs+1] fine-level counters (kept zero between steps)
    int* subOffset;             // [Cs+1] fine-level cell offsets
    int2* subKeySlot;           // [8n]
    int* subTmp;                // [8n]
    int* subSortedHash;         // [8n]
    int* subSortedIds;          // [8n] slots in (fine cell, list position) order
    float4* subPosS;            // [8n] child positions in that order
    float4* subVelS;            // [8n] child velocities in that order
    float splitMin[3], splitMax[3];
    int childMode;              // sph_options.childMode
};

// Per-row lookup tables of the neighbour search.
struct RowTables {
    const int* cellOffset;  // [C+1]
    const int* halfOffset;  // [C+1], valid for occupied cells
    const SceneDev* scenes; // batched handles: per-scene grids, constants, maps (else NULL)
    const int* skip;        // as SortBuffers::skip, read by the density stage only
};

// Reused neighbour lists (sph_options.neighbourSkin).  When the lists are
// built, every particle records the stencil rows of the reference grid that
// its skin sphere (radius R = (1 + skin) h) reaches: per row a window start
// in the working order and a 64-bit mask of the candidates within R.  Later
// steps keep that working order (the state is gathered into it) and visit
// only those candidates, until some particle has moved farther than 0.45 skin
// h from where it was at the build.  Slots 0-8 hold the reference's own 3 x 3
// rows in its order (an empty row: start 0, no bits), so a build step sums
// exactly what the per-step search sums; the further rows the skin reaches
// follow from slot 9.  A window whose candidates within R span more than 64
// places is kept unmasked: bit 31 of `start` set and the window end in the
// low word of its masks.
// Batched handles keep one set of flags per scene (field-major: field f of
// scene k at flags[f * numScenes + k]); each scene decides its builds from
// its own particles' displacement and its own h, so a scene in a batch
// builds exactly when it would alone.  The list kernels take a slot's scene
// from slotScene (the .w lane of the sorted position, which carries the
// scene in the batch's other kernels, holds p/rho^2 once a list density
// kernel has run).
constexpr int VL_SLOTS = 16;  // rows within R <= 1.4 gridSpacing: at most 4 x 4
constexpr int VL_INNER = 9;
enum : int {
    VL_BUILD = 0,      // a build is requested (state written, another kind of step ran)
    VL_BUILD_NOW = 1,  // this step builds the lists (decided at the start of the step)
    VL_DISP = 2,       // largest squared displacement since the build (float bits)
    VL_COUNT = 3,      // builds so far
    VL_FLAGS = 4,
};
// Two words after the per-scene flags: whether this step sorts (some scene
// builds; a step that builds nothing keeps the working order and skips the
// hash, scan and scatter), and whether the cell tables on the device are
// older than the last step (it skipped them; sph_read_cells rebuilds them
// from that step's sorted copies).
enum : int { VL_SORT = 0, VL_STALE = 1, VL_GLOBAL = 2 };
struct NeighbourLists {
    int* start;            // [VL_SLOTS][n] window start (bit 31: unmasked window)
    uint2* skin;           // [VL_SLOTS][n] candidates within R (bit k: start + k; .x bits 0-31), or
                           //               .x = the window end
    uint2* exact;          // [VL_SLOTS][n] this step's neighbours (0 < r <= h) over the same window, or
                           //               .x = the window end
    unsigned char* rows;   // [n] slots in use (9 + the further rows)
    float4* posB;          // [n] positions at the build, working order
    unsigned int* flags;   // [VL_FLAGS][numScenes], then [VL_GLOBAL]
    float radius, radius2; // R and R^2 (single-scene handles; a batch's kernels take each scene's h)
    float dispLimit2;      // (0.45 skin h)^2 (likewise)
    float skinFrac;        // sph_options.neighbourSkin
    int numScenes;         // 1, or the batch's scene count
    int* slotScene;        // batched handles: [n] the scene of each sorted slot (a scene's particles
                           // always fill the same slot range: its cells follow the previous scene's)
};

// Launch configuration of the step (chosen per handle; see the autotuner).
enum ForceVariant { FORCE_DIRECT = 0, FORCE_MASK = 1, FORCE_PRETESTED = 2, FORCE_STAGED = 3 };

struct StepConfig {
    int densityBlock = 128;
    int forceBlock = 128;
    int forceVariant = FORCE_PRETESTED;
    int prune = 1;   // row / half-cell window cut (sph_device.cuh)
    int kahan = 1;
};

// Raises a kernel's dynamic shared memory limit once per device (the
// attribute belongs to the current device); K is the kernel itself, so each
// kernel keeps its own record.
template <auto K>
inline void ensure_dynamic_smem(int bytes) {
    static unsigned long long done = 0ull;  // one bit per device ordinal below 64
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = dev < 64 ? 1ull << dev : 0ull;
    if (bit && (done & bit)) return;
    if (cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess) done |= bit;
}

// The current device's multiprocessor count.
inline int device_sms() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 32;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// ---------------------------------------------------------------------------
// Launch wrappers (sph_kernels.cu)
// ---------------------------------------------------------------------------
void launch_unpack_aos(const float* aos, int stride, int offset, int n, float4* out, cudaStream_t s);
// pos[i].w = scene index `sid` (as integer bits) for i < count.
void launch_set_scene(float4* pos, int count, int sid, cudaStream_t s);
void launch_pack_aos(const float4* in, int n, float* aos, int stride, int offset, cudaStream_t s);
// Cell-relative positions: absolute -> (offset, packed cell) in place, and
// back to absolute (AoS with `stride` floats per particle and/or float4s).
void launch_abs_to_rel(int n, float4* pos, GridDev g, cudaStream_t s);
void launch_rel_to_abs(int n, const float4* pos, GridDev g, float* aos, int stride, float4* out4, cudaStream_t s);
// With `lists`, a one-block kernel first decides whether each scene builds
// the neighbour lists in this step (VL_BUILD_NOW) and whether the step sorts
// (VL_SORT); the hash pass returns at once when it does not.
void launch_hash_count(int n, const float4* pos, GridDev g, SortBuffers sb, unsigned int* status,
                       cudaStream_t s, const NeighbourLists* lists = nullptr);
// With `lists`, the scan and the scatter return at once in a step that
// builds no lists (VL_SORT clear), and so does the hash pass (whose checks of
// the state the rank pass then makes).
void launch_cell_scan(int numCells, SortBuffers sb, unsigned int* status, cudaStream_t s,
                      const NeighbourLists* lists = nullptr);
// With `status`, the scatter leaves its outputs as they were once a scan
// wait has given up (STATUS_DEVICE_WAIT).
void launch_scatter(int n, SortBuffers sb, cudaStream_t s, const unsigned int* status = nullptr,
                    const NeighbourLists* lists = nullptr);
// The cell tables of the sorted copies' positions (sortedHash, sortedIds,
// cellOffset) after a step that skipped them; the working order, the sorted
// copies and the lists stay as they are.  `scratch`: n float4.
void launch_rebuild_tables(int n, const float4* posS, const int* workIds, const int* slotScene, GridDev g,
                           SortBuffers sb, float4* scratch, unsigned int* status, cudaStream_t s);
// With `lists` and no build in this step, only the reference permutation is
// ranked and the state is gathered into the kept working order (workIds).
// With `status`, the pass leaves its outputs as they were once a scan wait
// has given up (STATUS_DEVICE_WAIT).
// In a step that sorts nothing (lists, VL_SORT clear) the pass only gathers
// the state into the kept order and makes the hash pass's checks (non-finite
// positions, positions outside the grid), latching them in `status`.
void launch_rank_gather(int n, SortBuffers sb, const float4* pos, const float4* vel, GridDev g,
                        float4* posS, float4* velS, cudaStream_t s, const NeighbourLists* lists = nullptr,
                        unsigned int* status = nullptr);
// Density stage over reused neighbour lists: the build form (the reference's
// rows and the skin rows, recording the lists) and the list form; each
// returns at once unless the step is of its kind.
// Besides rho4S, each particle's p/rho^2 and 1/rho go to the fourth lanes of
// its sorted position and velocity, where the list force stage reads them.
void launch_density_lists(int n, float4* posS, float4* velS, RowTables T, GridDev g, PhysDev ph, MapDev map,
                          float4* rho4S, const NeighbourLists& L, const StepConfig& cfg, bool build, bool reuse,
                          cudaStream_t s);
// After a write of the positions: the largest distance from the build
// positions, measured afresh (the lists stay if it is within the limit).
// (Batched handles: each particle's scene from the .w lane of its position.)
void launch_list_displacement(int n, const float4* pos, const int* workIds, const NeighbourLists& L,
                              cudaStream_t s);
// Force stage over the lists' neighbour masks; also records the largest
// displacement since the build.  With `scenes` (batched handles) each
// particle's constants and maps come from its scene's record.
void launch_force_lists(int n, const float4* posS, const float4* velS, const float4* rho4S, const int* workIds,
                        PhysDev ph, MapDev map, int collide, const NeighbourLists& L, float4* pos, float4* vel,
                        float4* accS, const StepConfig& cfg, cudaStream_t s, const SceneDev* scenes = nullptr);
void launch_density(int n, const float4* posS, RowTables T, GridDev g, PhysDev ph, MapDev map,
                    float4* rho4S, int* rowStart, unsigned int* rowMask, const StepConfig& cfg,
                    cudaStream_t s);
// Learned-step features recorded by the force stage (24 floats per particle
// at index workIds[i] when byId, else i; see feature_values in sph_step.cu).
struct FeatureOut {
    float* feat;
    int byId;
    int boxWalls;
    float dtL;
};
void launch_force(int n, const float4* posS, const float4* velS, const float4* rho4S,
                  const int* workIds, RowTables T, GridDev g, PhysDev ph, MapDev map, int collide,
                  const int* rowStart, const unsigned int* rowMask, float4* pos, float4* vel,
                  float4* accS, const StepConfig& cfg, cudaStream_t s, const FeatureOut* feat = nullptr,
                  unsigned int* status = nullptr);
void launch_unpermute(int n, const int* sortedIds, const float4* srcS, int comp, float* dst,
                      int stride, int offset, cudaStream_t s);
void launch_cell_tables(int numCells, const int* cellOffset, int* start, int* end, cudaStream_t s);

// Two-scale pass (sph_twoscale.cu).
void launch_ts_states(int n, const float4* posS, const int* workIds, const int* cellOffset, GridDev g, float h,
                      const TwoScaleDev& T, cudaStream_t s);
void launch_ts_children(int n, float4* posS, float4* velS, const float4* accS, const float4* rho4S,
                        const int* workIds, float mass, PhysDev ph, int collide, float4* pos, float4* vel,
                        const TwoScaleDev& T, cudaStream_t s);
void launch_ts_project(const float4* coarsePos, const int* workIds, int byId, const float4* rho4S,
                       const int* cellOffset, GridDev g, float hs, const TwoScaleDev& T, int capacity,
                       cudaStream_t s);
void launch_ts_sub_sort(GridDev sg, const TwoScaleDev& T, SortBuffers subSb, int capacity, unsigned int* status,
                        cudaStream_t s);
void launch_ts_sub_density(GridDev sg, PhysDev sph, const TwoScaleDev& T, int capacity, cudaStream_t s);
void launch_ts_sub_force(GridDev sg, PhysDev sph, const TwoScaleDev& T, int capacity, cudaStream_t s);
void launch_ts_pack_sd(const TwoScaleDev& T, int slots, float* dst, cudaStream_t s);

// FP64 diagnostics (sph_diag.cu): out[DIAG_TERMS] in this order; the maximum
// relative density error is the last term.
enum { DIAG_MASS = 0, DIAG_MOM_X, DIAG_MOM_Y, DIAG_MOM_Z, DIAG_KINETIC, DIAG_POTENTIAL, DIAG_RHO_SUM,
       DIAG_RHO_MAXERR, DIAG_TERMS };
int diag_partial_rows();
void launch_diagnostics(int n, const float4* pos, const float4* vel, const float4* rho4S, int haveRho,
                        double mass, double gravity, double rest0, int axis, double* partial, double* out,
                        cudaStream_t s);

// Boundary maps.
// Builds the maps of `d` (grid solids are uploaded for the build and freed
// after it, synchronising `s`).
cudaError_t launch_build_maps(const sph_boundary_desc& d, const unsigned int dims[3], float* dist,
                              float* dens, float* visc, float4* map4, cudaStream_t s);

}  // namespace sph
