// Host harness that runs the reference's own SPH step code on the CPU.
//
// Test infrastructure (the oracle), never part of the product.  The
// reference's device functions and kernels of the plain step are taken
// verbatim, at build time, from its particle_simulation.cu (and its
// SimulationParameters / VD / SD declarations from particle_simulation.h) by
// oracle/build_ref.py, which writes them to oracle/_ref/ref_types.inc and
// oracle/_ref/ref_funcs.inc; nothing of the reference is kept in this
// repository.  This file supplies what those functions expect of CUDA:
//   * float3 / int3 and the __device__, __global__ qualifiers;
//   * blockIdx / blockDim / threadIdx (one copy per host thread), set by the
//     launch loop below, which runs a kernel's threads over the host's cores
//     with OpenMP (every kernel used here writes only its own thread's
//     outputs and reads only what earlier kernels wrote, as on the GPU);
//   * tex1Dfetch over the arrays the reference binds to its 1-D textures
//     (particle_simulation.cu:28-39, bound at :1979-1994);
//   * tex3D with the documented normalised, linear, clamped addressing of
//     its boundary-map textures (set_up_3d_float_texture, :2959-3011), with
//     exact FP32 weights (the hardware's 9-bit weights are not restated);
//   * the __constant__ parameters (gSimParamsDev, gBoundary*).
// The step follows Advance (particle_simulation.cu:2085-2117) plus the
// handleCollisions of AdvanceTwoScale (:2170): hash (compute_particle_hash,
// the reference's kernel), sort by hash (restated: a stable sort, the
// semantics of the thrust::sort_by_key call at :2340), cell start/end
// (restated from compute_cell_start_end, :155-193, whose two shared-memory
// phases cannot run one thread at a time; empty cells hold 0xFFFFFFFF as the
// memsets at :2362-2363 leave them), density (compute_particle_density_pressure,
// the reference's kernel), forces (compute_particle_acceleration_ifsurf),
// integrate_euler and, when asked, collision_handling -- all the reference's.
// Compiled for the host with -ffp-contract=off (no fused multiply-add: nvcc
// would fuse some products and sums on the GPU, so results agree with the
// GPU reference to FP32 rounding, not bit for bit) and with uninitialised
// locals zeroed (compute_particle_acceleration_ifsurf reads colLapl before
// writing it, :381; the build of this repository starts it at 0 too).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using std::abs;
using std::max;
using std::min;
using std::sqrt;

#define __device__
#define __global__
#define __host__
#define __constant__ static

struct float3 {
    float x, y, z;
};
struct int3 {
    int x, y, z;
};
struct dim3 {
    unsigned int x = 0, y = 0, z = 0;
};
static thread_local dim3 blockIdx, blockDim, threadIdx;

// The reference's texture references become plain arrays.
template <class T>
struct Tex1D {
    const T* data = nullptr;
};
template <class T>
static inline T tex1Dfetch(const Tex1D<T>& t, int i) {
    return t.data[i];
}

struct Tex3D {
    const float* data = nullptr;  // x fastest
    int dims[3] = {0, 0, 0};
};

// Normalised coordinates, linear filter, clamp addressing: texel coordinate
// u * N - 0.5 per axis, the two nodes around it clamped to [0, N - 1], and
// the blend v0 + a (v1 - v0) along x, then y, then z.  No map bound: 0.
static inline float tex3D(const Tex3D& t, float u, float v, float w) {
    if (!t.data) return 0.0f;
    const float c[3] = {u, v, w};
    int i0[3], i1[3];
    float a[3];
    for (int k = 0; k < 3; k++) {
        const float x = c[k] * (float)t.dims[k] - 0.5f;
        const float f = std::floor(x);
        a[k] = x - f;
        const long long lo = (long long)f;
        i0[k] = (int)std::min<long long>(std::max<long long>(lo, 0), t.dims[k] - 1);
        i1[k] = (int)std::min<long long>(std::max<long long>(lo + 1, 0), t.dims[k] - 1);
    }
    auto at = [&](int x, int y, int z) {
        return t.data[(size_t)x + (size_t)t.dims[0] * ((size_t)y + (size_t)t.dims[1] * (size_t)z)];
    };
    auto lerp = [](float p, float q, float s) { return p + s * (q - p); };
    const float c00 = lerp(at(i0[0], i0[1], i0[2]), at(i1[0], i0[1], i0[2]), a[0]);
    const float c10 = lerp(at(i0[0], i1[1], i0[2]), at(i1[0], i1[1], i0[2]), a[0]);
    const float c01 = lerp(at(i0[0], i0[1], i1[2]), at(i1[0], i0[1], i1[2]), a[0]);
    const float c11 = lerp(at(i0[0], i1[1], i1[2]), at(i1[0], i1[1], i1[2]), a[0]);
    return lerp(lerp(c00, c10, a[1]), lerp(c01, c11, a[1]), a[2]);
}

// enums and SimulationParameters of particle_simulation.h
#include "_ref/ref_types.inc"

// the reference's constant memory and texture bindings
static SimulationParameters gSimParamsDev;
static Tex1D<float> gParticleVertexData, gParticleSimulationData;
static Tex1D<int> gCellStartList, gCellEndList, gSortedParticleIdList, gParticleHashList;
static float gBoundaryGridOrigin[3];
static float gBoundaryGridSpacing;
static unsigned int gBoundaryGridDimensions[3];
static float gBoundaryGridLength[3];
static float gBoundaryRestDistance;
static Tex3D gBoundaryDistances, gBoundaryDensities, gBoundaryViscosities;

// the reference's device functions and kernels of the plain step
#include "_ref/ref_funcs.inc"

// Runs kernel() for `n` threads in blocks of 256, spread over the host's cores.
template <class F>
static void launch(unsigned int n, F&& kernel) {
#pragma omp parallel for schedule(static)
    for (long long idx = 0; idx < (long long)n; idx++) {
        blockDim.x = 256;
        blockIdx.x = (unsigned int)(idx / 256);
        threadIdx.x = (unsigned int)(idx % 256);
        kernel();
    }
}

extern "C" {

void ref_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

// One plain step of the reference's code.  params: a SimulationParameters
// image (180 bytes, the layout of particle_simulation.h:54-111).  vd: float[n*3]
// positions, sd: float[n*10] simulation data (velocities in SD_VEL0_*),
// both updated in place.  Boundary maps (distance, density, viscosity on a
// dims[0] x dims[1] x dims[2] grid, x fastest) may be NULL, in which case the
// wall terms read 0 as from an unbound texture and restDistance is 0.
// Outputs: hash[n], ids[n] (sorted order), start[C], end[C].
int ref_step_plain(const void* params, float* vd, float* sd, const float* mapDist, const float* mapDens,
                   const float* mapVisc, const unsigned int* mapDims, const float* mapOrigin, float mapSpacing,
                   float restDistance, int collide, int* hash, int* ids, int* start, int* end) {
    std::memcpy(&gSimParamsDev, params, sizeof(SimulationParameters));
    const unsigned int n = gSimParamsDev.numParticles;
    const int C = gSimParamsDev.gridDim[0] * gSimParamsDev.gridDim[1] * gSimParamsDev.gridDim[2];
    gParticleVertexData.data = vd;
    gParticleSimulationData.data = sd;
    gBoundaryDistances = Tex3D{};
    gBoundaryDensities = Tex3D{};
    gBoundaryViscosities = Tex3D{};
    gBoundaryRestDistance = 0.0f;
    for (int a = 0; a < 3; a++) {
        gBoundaryGridOrigin[a] = 0.0f;
        gBoundaryGridLength[a] = 1.0f;
        gBoundaryGridDimensions[a] = 0;
    }
    gBoundaryGridSpacing = 1.0f;
    if (mapDist && mapDens && mapVisc && mapDims && mapOrigin) {
        // setUpSphInComplexShapes (particle_simulation.cu:2592-2683): origin,
        // spacing, dims, length = (dims - 1) * spacing, rest distance
        for (int a = 0; a < 3; a++) {
            gBoundaryGridOrigin[a] = mapOrigin[a];
            gBoundaryGridDimensions[a] = mapDims[a];
            gBoundaryGridLength[a] = (float)(mapDims[a] - 1) * mapSpacing;
        }
        gBoundaryGridSpacing = mapSpacing;
        gBoundaryRestDistance = restDistance;
        for (Tex3D* t : {&gBoundaryDistances, &gBoundaryDensities, &gBoundaryViscosities})
            for (int a = 0; a < 3; a++) t->dims[a] = (int)mapDims[a];
        gBoundaryDistances.data = mapDist;
        gBoundaryDensities.data = mapDens;
        gBoundaryViscosities.data = mapVisc;
    }

    // computeParticleHash
    std::vector<int> idList(n), hashList(n);
    launch(n, [&] { compute_particle_hash(vd, idList.data(), hashList.data(), n); });
    for (unsigned int i = 0; i < n; i++)
        if (hashList[i] < 0 || hashList[i] >= C) return 1;  // the reference would write outside its tables
    // sortParticleIdsByHash: stable by hash
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hashList[a] < hashList[b]; });
    for (unsigned int k = 0; k < n; k++) {
        hash[k] = hashList[order[k]];
        ids[k] = idList[order[k]];
    }
    // computeCellStartEndList
    std::fill(start, start + C, -1);
    std::fill(end, end + C, -1);
    for (unsigned int k = 0; k < n; k++) {
        if (k == 0 || hash[k] != hash[k - 1]) {
            start[hash[k]] = (int)k;
            if (k > 0) end[hash[k - 1]] = (int)k;
        }
        if (k == n - 1) end[hash[k]] = (int)k + 1;
    }
    gCellStartList.data = start;
    gCellEndList.data = end;
    gSortedParticleIdList.data = ids;
    gParticleHashList.data = hash;
    // computeParticleDensityPressure, computeParticleAcceleration, integrate
    launch(n, [&] { compute_particle_density_pressure(vd, sd, ids, start, end); });
    std::vector<int> surface(n, 0);
    launch(n, [&] { compute_particle_acceleration_ifsurf(vd, sd, ids, start, end, surface.data()); });
    launch(n, [&] { integrate_euler(vd, sd); });
    if (collide) launch(n, [&] { collision_handling(vd, sd); });
    return 0;
}

}  // extern "C"
