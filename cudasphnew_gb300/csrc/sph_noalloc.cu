// Neighbour-search tables without any device allocation.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// need the cell tables: a frame loop in which an allocation would synchronise
// the device and stall the frame, or an application that has handed its whole
// device memory budget to its own allocator up front.  For them,
// sph_cell_tables_noalloc() builds the same tables as sph_step() followed by
// sph_read_cells() -- sorted hashes, the sort permutation, cell start and end
// -- from positions and into output buffers the caller already owns, with all
// intermediate data in one file-scope device array of fixed size.
//
// That array is loaded with the library on every GPU that uses it and stays
// resident until the process exits.  Every call on a device shares it, and it
// keeps whatever the last call left there; the per-cell counters are cleared
// at the start of each call.  Calls whose work overlaps on the GPU (two
// streams, or two host threads, on the same device) race on the array and
// must be serialised by the caller.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress while that device is current; make that first call
// before any stream capture on that device.  Every call waits for its own
// work to finish (it reads the input-check flags back), so a call on a
// stream that is being captured is refused with SPH_ERR_NOT_SUPPORTED before
// anything is enqueued.
//
// Cost: the stable order inside a cell compares every particle of the cell
// with every other (k^2 work for a cell of k particles).  At a few particles
// per cell that is nothing, but positions crowded into one cell make it
// quadratic: 65,536 particles in one cell take about 4e9 comparisons (seconds).
// Inputs that fail the checks (non-finite or outside the grid) skip that pass.
#include <mutex>
#include <string>

#include "sph_device.cuh"

namespace {

constexpr int NA_MAX_PARTICLES = SPH_NOALLOC_MAX_PARTICLES;
constexpr int NA_MAX_CELLS = SPH_NOALLOC_MAX_CELLS;
constexpr int NA_SCAN_THREADS = 1024;

// Scratch layout (bytes):
//   flags    unsigned int (+ padding to 256 B)  out-of-range / non-finite input
//   counts   int[NA_MAX_CELLS + 1]   per-cell arrival counters
//   offsets  int[NA_MAX_CELLS + 1]   their exclusive scan
//   keySlot  int2[NA_MAX_PARTICLES]  (hash, arrival slot)
//   tmpIds   int[NA_MAX_PARTICLES]   ids in their cell segment, unordered
constexpr size_t NA_FLAGS = 0;
constexpr size_t NA_COUNTS = 256;
constexpr size_t NA_OFFSETS = NA_COUNTS + sizeof(int) * ((size_t)NA_MAX_CELLS + 64);
constexpr size_t NA_KEYSLOT = NA_OFFSETS + sizeof(int) * ((size_t)NA_MAX_CELLS + 64);
constexpr size_t NA_TMPIDS = NA_KEYSLOT + sizeof(int2) * (size_t)NA_MAX_PARTICLES;
constexpr size_t NA_BYTES = NA_TMPIDS + sizeof(int) * (size_t)NA_MAX_PARTICLES;

static __device__ __align__(256) unsigned char g_naScratch[NA_BYTES];

struct NaView {
    unsigned int* flags;
    int* counts;
    int* offsets;
    int2* keySlot;
    int* tmpIds;
};

inline NaView na_view(unsigned char* base) {
    return NaView{reinterpret_cast<unsigned int*>(base + NA_FLAGS), reinterpret_cast<int*>(base + NA_COUNTS),
                  reinterpret_cast<int*>(base + NA_OFFSETS), reinterpret_cast<int2*>(base + NA_KEYSLOT),
                  reinterpret_cast<int*>(base + NA_TMPIDS)};
}

// Everything that must start at zero: the counters and the flags.
__global__ void k_na_clear(NaView v, int total) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < total) v.counts[c] = 0;
    if (c == 0) *v.flags = 0u;
}

// compute_particle_hash (particle_simulation.cu:89-119) on the reference's VD
// layout (three floats per particle), plus the arrival slot in the cell.
__global__ void k_na_hash(int n, const float* __restrict__ vd, sph::GridDev g, NaView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = make_float4(vd[3 * (size_t)i], vd[3 * (size_t)i + 1], vd[3 * (size_t)i + 2], 0.f);
    bool outside = false;
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) {
        atomicOr(v.flags, 2u);
        p = make_float4(g.origin[0], g.origin[1], g.origin[2], 0.f);
    }
    int h = sph::particle_hash(p, g, &outside);
    if (outside) atomicOr(v.flags, 1u);
    v.keySlot[i] = make_int2(h, atomicAdd(v.counts + h, 1));
}

// Exclusive scan of total counters by one block (the sizes here are modest).
__global__ void __launch_bounds__(NA_SCAN_THREADS) k_na_scan(NaView v, int total) {
    __shared__ int s_warp[NA_SCAN_THREADS / 32];
    __shared__ int s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < total; base += NA_SCAN_THREADS) {
        const int idx = base + threadIdx.x;
        const int x = idx < total ? v.counts[idx] : 0;
        int incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        const int excl = s_carry + (warp > 0 ? s_warp[warp - 1] : 0) + incl - x;
        if (idx < total) v.offsets[idx] = excl;
        __syncthreads();
        if (threadIdx.x == NA_SCAN_THREADS - 1) s_carry = excl + x;
        __syncthreads();
    }
}

__global__ void k_na_scatter(int n, NaView v, int* __restrict__ sortedHash) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int2 ks = v.keySlot[i];
    int dst = v.offsets[ks.x] + ks.y;
    v.tmpIds[dst] = i;
    sortedHash[dst] = ks.x;
}

// Stable order inside each cell: rank = number of smaller ids in the segment.
// Skipped when the input checks failed: the call returns an error then, and
// inputs clamped into one cell would make this pass quadratic in n.
__global__ void k_na_rank(int n, NaView v, const int* __restrict__ sortedHash, int* __restrict__ sortedIds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || *v.flags) return;
    int c = sortedHash[k];
    int s = v.offsets[c], e = v.offsets[c + 1];
    int my = v.tmpIds[k];
    int r = 0;
    for (int t = s; t < e; t++) r += v.tmpIds[t] < my;
    sortedIds[s + r] = my;
}

// Cell start/end with 0xFFFFFFFF for empty cells (compute_cell_start_end and
// its memsets, particle_simulation.cu:155-193, 2357-2369).
__global__ void k_na_tables(int numCells, NaView v, int* __restrict__ start, int* __restrict__ end) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCells) return;
    int s = v.offsets[c], e = v.offsets[c + 1];
    bool occ = e > s;
    start[c] = occ ? s : -1;
    end[c] = occ ? e : -1;
}

// Per-device address of g_naScratch, looked up once with that device current.
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_naMutex;
unsigned char* g_naBase[NA_MAX_DEVICES] = {};

}  // namespace

namespace sph {
sph_status record_error(sph_status st, const char* file, int line, const std::string& msg);
}

#define NA_FAIL(st, msg) return sph::record_error((st), __FILE__, __LINE__, (msg))

extern "C" sph_status sph_cell_tables_noalloc(const SimulationParameters* params, const float* devVertexData,
                                              unsigned int n, int* devSortedHash, int* devSortedIds,
                                              int* devCellStart, int* devCellEnd, void* stream) {
    if (!params || !devVertexData || !devSortedHash || !devSortedIds || !devCellStart || !devCellEnd)
        NA_FAIL(SPH_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0 || n > (unsigned int)NA_MAX_PARTICLES)
        NA_FAIL(SPH_ERR_INVALID_ARGUMENT,
                "n must be in [1, SPH_NOALLOC_MAX_PARTICLES = " + std::to_string(NA_MAX_PARTICLES) + "]");
    double cells = 1.0;
    for (int a = 0; a < 3; a++) {
        if (params->gridDim[a] <= 0) NA_FAIL(SPH_ERR_INVALID_ARGUMENT, "gridDim must be positive");
        cells *= params->gridDim[a];
    }
    if (cells > (double)NA_MAX_CELLS)
        NA_FAIL(SPH_ERR_INVALID_ARGUMENT, "gridDim[0]*gridDim[1]*gridDim[2] exceeds SPH_NOALLOC_MAX_CELLS = " +
                                              std::to_string(NA_MAX_CELLS));
    if (!(params->gridSpacing > 0.0f)) NA_FAIL(SPH_ERR_INVALID_ARGUMENT, "gridSpacing must be positive");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) NA_FAIL(SPH_ERR_CUDA, cudaGetErrorString(e));
    if (cap != cudaStreamCaptureStatusNone)
        NA_FAIL(SPH_ERR_NOT_SUPPORTED, "the stream is being captured: this call waits for its own work");
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) NA_FAIL(SPH_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= NA_MAX_DEVICES) NA_FAIL(SPH_ERR_NOT_SUPPORTED, "device index too large");
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_naMutex);
        if (!g_naBase[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_naScratch);
            if (e != cudaSuccess) NA_FAIL(SPH_ERR_CUDA, cudaGetErrorString(e));
            g_naBase[dev] = static_cast<unsigned char*>(p);
        }
        base = g_naBase[dev];
    }
    sph::GridDev g;
    for (int a = 0; a < 3; a++) {
        g.origin[a] = params->gridOrigin[a];
        g.dim[a] = params->gridDim[a];
    }
    g.spacing = params->gridSpacing;
    g.numCells = g.dim[0] * g.dim[1] * g.dim[2];
    g.cellBase = 0;
    const NaView v = na_view(base);
    const int total = g.numCells + 1;
    const int nn = (int)n;
    k_na_clear<<<(total + 255) / 256, 256, 0, st>>>(v, total);
    k_na_hash<<<(nn + 255) / 256, 256, 0, st>>>(nn, devVertexData, g, v);
    k_na_scan<<<1, NA_SCAN_THREADS, 0, st>>>(v, total);
    k_na_scatter<<<(nn + 255) / 256, 256, 0, st>>>(nn, v, devSortedHash);
    k_na_rank<<<(nn + 255) / 256, 256, 0, st>>>(nn, v, devSortedHash, devSortedIds);
    k_na_tables<<<(g.numCells + 255) / 256, 256, 0, st>>>(g.numCells, v, devCellStart, devCellEnd);
    e = cudaGetLastError();
    if (e != cudaSuccess) NA_FAIL(SPH_ERR_CUDA, cudaGetErrorString(e));
    unsigned int flags = 0;
    e = cudaMemcpyAsync(&flags, v.flags, sizeof(flags), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) NA_FAIL(SPH_ERR_CUDA, cudaGetErrorString(e));
    if (flags & 2u) NA_FAIL(SPH_ERR_NON_FINITE, "a non-finite particle position was given");
    if (flags & 1u) NA_FAIL(SPH_ERR_OUT_OF_DOMAIN, "a particle was hashed outside the cell grid");
    return SPH_OK;
}
