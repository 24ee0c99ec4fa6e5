// Kernels of the GB300 SPH step (sm_103a).
//
// Data layout in HBM (one handle, n particles, C cells):
//   pos, vel           float4[n]  particle-index order (the state; .w unused)
//   posS, velS         float4[n]  copies in sorted (cell, id) order, per step
//   rho4S              float4[n]  (rho, p, p/rho^2, 1/rho) in sorted order
//   accS               float4[n]  acceleration in sorted order
//   cnt, cellOffset    int[C+1]   per-cell counts / their exclusive scan
// The sort is a counting sort: every particle takes an arrival slot in its
// cell with one atomic, a single-pass decoupled look-back scan turns counts
// into cell offsets, and a rank pass orders each cell's members by particle
// id.  The result is the permutation of a stable sort by hash -- the order
// thrust::sort_by_key produces in the reference (particle_simulation.cu:2340).
#include <cuda/atomic>

#include "sph_internal.h"

namespace sph {

// ---------------------------------------------------------------------------
// Reference grid arithmetic, bit-exact
// ---------------------------------------------------------------------------

// compute_particle_hash (particle_simulation.cu:100-115): (int) truncation,
// C remainder, x-fastest hash.  Rounded operations are spelled out so no FMA
// contraction can change the cell a particle falls in.
__device__ __forceinline__ int particle_hash(float4 p, const GridDev& g, bool* outside) {
    int c[3];
    float v[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float f = __fdiv_rn(__fsub_rn(v[a], g.origin[a]), g.spacing);
        c[a] = (int)f;
        c[a] = c[a] % g.dim[a];
    }
    int h = g.dim[0] * (g.dim[1] * c[2] + c[1]) + c[0];
    if (h < 0 || h >= g.numCells) {
        *outside = true;
        h = min(max(h, 0), g.numCells - 1);
    }
    return h;
}

// compute_grid_coordinate (particle_simulation.cu:1238-1258): the (unsigned)
// conversion saturates negative values to 0, then remainder and clamp.
__device__ __forceinline__ int grid_coord(float p, float d, float origin, float spacing, int dim) {
    float f = __fdiv_rn(__fsub_rn(__fadd_rn(p, d), origin), spacing);
    unsigned int u = (unsigned int)f;
    int c = (int)u;
    c = c % dim;
    return min(max(c, 0), dim - 1);
}

// ---------------------------------------------------------------------------
// Software trilinear fetch with CUDA's normalised-coordinate addressing
// (texel coordinate u*N - 0.5, clamp), exact FP32 weights.
// ---------------------------------------------------------------------------
struct Tri {
    int i0[3], i1[3];
    float a[3];
};

__device__ __forceinline__ Tri tri_setup(const MapDev& m, float u, float v, float w) {
    Tri t;
    float c[3] = {u, v, w};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float x = __fsub_rn(__fmul_rn(c[k], m.dimsf[k]), 0.5f);
        float f = floorf(x);
        t.a[k] = __fsub_rn(x, f);
        int lo = (int)f;  // saturating; |x| is small for in-range particles
        t.i0[k] = min(max(lo, 0), m.dims[k] - 1);
        t.i1[k] = min(max(lo + 1, 0), m.dims[k] - 1);
    }
    return t;
}

// v0 + a*(v1 - v0): exact for a constant field, so the clamped region of the
// distance map (-restDistance everywhere) never trips the wall test.
__device__ __forceinline__ float lerp_ref(float v0, float v1, float a) {
    return __fadd_rn(v0, __fmul_rn(a, __fsub_rn(v1, v0)));
}

__device__ __forceinline__ size_t node(const MapDev& m, int x, int y, int z) {
    return (size_t)x + (size_t)m.dims[0] * ((size_t)y + (size_t)m.dims[1] * (size_t)z);
}

__device__ __forceinline__ float tri_scalar(const MapDev& m, const float* __restrict__ g, float u,
                                            float v, float w) {
    Tri t = tri_setup(m, u, v, w);
    float c00 = lerp_ref(__ldg(g + node(m, t.i0[0], t.i0[1], t.i0[2])),
                         __ldg(g + node(m, t.i1[0], t.i0[1], t.i0[2])), t.a[0]);
    float c10 = lerp_ref(__ldg(g + node(m, t.i0[0], t.i1[1], t.i0[2])),
                         __ldg(g + node(m, t.i1[0], t.i1[1], t.i0[2])), t.a[0]);
    float c01 = lerp_ref(__ldg(g + node(m, t.i0[0], t.i0[1], t.i1[2])),
                         __ldg(g + node(m, t.i1[0], t.i0[1], t.i1[2])), t.a[0]);
    float c11 = lerp_ref(__ldg(g + node(m, t.i0[0], t.i1[1], t.i1[2])),
                         __ldg(g + node(m, t.i1[0], t.i1[1], t.i1[2])), t.a[0]);
    return lerp_ref(lerp_ref(c00, c10, t.a[1]), lerp_ref(c01, c11, t.a[1]), t.a[2]);
}

__device__ __forceinline__ float4 lerp4(float4 p, float4 q, float a) {
    return make_float4(lerp_ref(p.x, q.x, a), lerp_ref(p.y, q.y, a), lerp_ref(p.z, q.z, a), 0.f);
}

__device__ __forceinline__ float4 tri_vec(const MapDev& m, float u, float v, float w) {
    Tri t = tri_setup(m, u, v, w);
    const float4* g = m.map4;
    float4 c00 = lerp4(__ldg(g + node(m, t.i0[0], t.i0[1], t.i0[2])),
                       __ldg(g + node(m, t.i1[0], t.i0[1], t.i0[2])), t.a[0]);
    float4 c10 = lerp4(__ldg(g + node(m, t.i0[0], t.i1[1], t.i0[2])),
                       __ldg(g + node(m, t.i1[0], t.i1[1], t.i0[2])), t.a[0]);
    float4 c01 = lerp4(__ldg(g + node(m, t.i0[0], t.i0[1], t.i1[2])),
                       __ldg(g + node(m, t.i1[0], t.i0[1], t.i1[2])), t.a[0]);
    float4 c11 = lerp4(__ldg(g + node(m, t.i0[0], t.i1[1], t.i1[2])),
                       __ldg(g + node(m, t.i1[0], t.i1[1], t.i1[2])), t.a[0]);
    return lerp4(lerp4(c00, c10, t.a[1]), lerp4(c01, c11, t.a[1]), t.a[2]);
}

__device__ __forceinline__ void map_uvw(const MapDev& m, float4 x, float* uvw) {
    uvw[0] = __fdiv_rn(__fsub_rn(x.x, m.origin[0]), m.length[0]);
    uvw[1] = __fdiv_rn(__fsub_rn(x.y, m.origin[1]), m.length[1]);
    uvw[2] = __fdiv_rn(__fsub_rn(x.z, m.origin[2]), m.length[2]);
}

// ---------------------------------------------------------------------------
// AoS <-> float4 conversion (VD/SD layouts of particle_simulation.h:17-41)
// ---------------------------------------------------------------------------
__global__ void k_unpack_aos(const float* __restrict__ aos, int stride, int offset, int n,
                             float4* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = aos + (size_t)i * stride + offset;
    out[i] = make_float4(p[0], p[1], p[2], 0.0f);
}

__global__ void k_pack_aos(const float4* __restrict__ in, int n, float* __restrict__ aos, int stride,
                           int offset) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = in[i];
    float* p = aos + (size_t)i * stride + offset;
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

void launch_unpack_aos(const float* aos, int stride, int offset, int n, float4* out, cudaStream_t s) {
    if (n <= 0) return;
    k_unpack_aos<<<(n + 255) / 256, 256, 0, s>>>(aos, stride, offset, n, out);
}

void launch_pack_aos(const float4* in, int n, float* aos, int stride, int offset, cudaStream_t s) {
    if (n <= 0) return;
    k_pack_aos<<<(n + 255) / 256, 256, 0, s>>>(in, n, aos, stride, offset);
}

// ---------------------------------------------------------------------------
// Stage 1: hash + per-cell arrival slot
// ---------------------------------------------------------------------------
__global__ void k_hash_count(int n, const float4* __restrict__ pos, GridDev g, int* __restrict__ cnt,
                             int2* __restrict__ keySlot, unsigned int* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    bool outside = false;
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) {
        atomicOr(status, STATUS_NON_FINITE);
        p = make_float4(g.origin[0], g.origin[1], g.origin[2], 0.f);
    }
    int h = particle_hash(p, g, &outside);
    if (outside) atomicOr(status, STATUS_OUT_OF_DOMAIN);
    int slot = atomicAdd(cnt + h, 1);
    keySlot[i] = make_int2(h, slot);
}

void launch_hash_count(int n, const float4* pos, GridDev g, SortBuffers sb, unsigned int* status,
                       cudaStream_t s) {
    if (n <= 0) return;
    k_hash_count<<<(n + 255) / 256, 256, 0, s>>>(n, pos, g, sb.cnt, sb.keySlot, status);
}

// ---------------------------------------------------------------------------
// Stage 2: exclusive scan of the C+1 cell counts into cell offsets, one pass
// with decoupled look-back (Merrill & Garland).  Counts are cleared as they
// are read, ready for the next step.  Tiles take their index from an atomic
// counter, so every tile a block waits on has already started; each wait is
// bounded and latches STATUS_DEVICE_WAIT if it ever gives up.
// ---------------------------------------------------------------------------
constexpr unsigned long long FLAG_AGG = 1ull << 32;
constexpr unsigned long long FLAG_INC = 2ull << 32;
constexpr int SPIN_LIMIT = 1 << 22;

__global__ void __launch_bounds__(SCAN_THREADS)
k_cell_scan(int total, int* __restrict__ cnt, int* __restrict__ out, unsigned long long* flags,
            unsigned int* tileCounter, unsigned int* status) {
    __shared__ int s_tile;
    __shared__ int s_warp[SCAN_THREADS / 32];
    __shared__ int s_prefix;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(tileCounter, 1u);
    __syncthreads();
    const int tile = s_tile;
    const int base = tile * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    if (base + SCAN_ITEMS <= total) {
        int4 a = *reinterpret_cast<const int4*>(cnt + base);
        int4 b = *reinterpret_cast<const int4*>(cnt + base + 4);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        *reinterpret_cast<int4*>(cnt + base) = make_int4(0, 0, 0, 0);
        *reinterpret_cast<int4*>(cnt + base + 4) = make_int4(0, 0, 0, 0);
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            int idx = base + k;
            v[k] = idx < total ? cnt[idx] : 0;
            if (idx < total) cnt[idx] = 0;
        }
    }
    int local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) local += v[k];
    // block-wide exclusive scan of `local`
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < SCAN_THREADS / 32) s_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const int warpExcl = warp > 0 ? s_warp[warp - 1] : 0;
    const int aggregate = s_warp[SCAN_THREADS / 32 - 1];
    int excl = warpExcl + incl - local;

    // publish + look back (warp 0)
    if (warp == 0) {
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> mine(flags[tile]);
        if (lane == 0) {
            mine.store((tile == 0 ? FLAG_INC : FLAG_AGG) | (unsigned int)aggregate,
                       cuda::memory_order_release);
        }
        int prefix = 0;
        if (tile > 0) {
            int look = tile - 1;
            bool done = false;
            while (!done) {
                int t = look - lane;
                unsigned long long f = FLAG_INC;  // below tile 0: neutral, inclusive
                if (t >= 0) {
                    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> other(flags[t]);
                    int spins = 0;
                    f = other.load(cuda::memory_order_acquire);
                    while ((f >> 32) == 0ull) {
                        if (++spins > SPIN_LIMIT) {
                            atomicOr(status, STATUS_DEVICE_WAIT);
                            f = FLAG_INC;  // give up: treat as zero, result flagged
                            break;
                        }
                        __nanosleep(32);
                        f = other.load(cuda::memory_order_acquire);
                    }
                    if (t < 0) f = FLAG_INC;
                }
                unsigned int incMask = __ballot_sync(0xffffffffu, (f >> 32) == 2ull);
                int val = (int)(unsigned int)(f & 0xffffffffull);
                int first = incMask ? __ffs(incMask) - 1 : 32;  // nearest inclusive
                int contrib = lane <= first ? val : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
                prefix += contrib;
                if (incMask) done = true;
                look -= 32;
            }
            if (lane == 0)
                mine.store(FLAG_INC | (unsigned int)(prefix + aggregate), cuda::memory_order_release);
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    int run = s_prefix + excl;
    if (base + SCAN_ITEMS <= total) {
        int o[SCAN_ITEMS];
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            o[k] = run;
            run += v[k];
        }
        *reinterpret_cast<int4*>(out + base) = make_int4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<int4*>(out + base + 4) = make_int4(o[4], o[5], o[6], o[7]);
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            if (base + k < total) out[base + k] = run;
            run += v[k];
        }
    }
}

void launch_cell_scan(int numCells, SortBuffers sb, unsigned int* status, cudaStream_t s) {
    int total = numCells + 1;
    int tiles = (total + SCAN_TILE - 1) / SCAN_TILE;
    // tile counter (first 16 bytes) and the tile states that follow it
    cudaMemsetAsync(sb.tileCounter, 0, 16 + sizeof(unsigned long long) * (size_t)tiles, s);
    k_cell_scan<<<tiles, SCAN_THREADS, 0, s>>>(total, sb.cnt, sb.cellOffset, sb.scanFlags,
                                               sb.tileCounter, status);
}

// ---------------------------------------------------------------------------
// Stage 3: scatter ids into their cell segments (arrival order)
// ---------------------------------------------------------------------------
__global__ void k_scatter(int n, const int2* __restrict__ keySlot, const int* __restrict__ cellOffset,
                          int* __restrict__ tmpIds, int* __restrict__ sortedHash) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int2 ks = keySlot[i];
    int dst = __ldg(cellOffset + ks.x) + ks.y;
    tmpIds[dst] = i;
    sortedHash[dst] = ks.x;
}

void launch_scatter(int n, SortBuffers sb, cudaStream_t s) {
    if (n <= 0) return;
    k_scatter<<<(n + 255) / 256, 256, 0, s>>>(n, sb.keySlot, sb.cellOffset, sb.tmpIds, sb.sortedHash);
}

// ---------------------------------------------------------------------------
// Stage 4: order each cell's members by id (rank = number of smaller ids in
// the segment) and gather the state into sorted order.
// ---------------------------------------------------------------------------
__global__ void k_rank_gather(int n, const int* __restrict__ sortedHash, const int* __restrict__ cellOffset,
                              const int* __restrict__ tmpIds, const float4* __restrict__ pos,
                              const float4* __restrict__ vel, int* __restrict__ sortedIds,
                              float4* __restrict__ posS, float4* __restrict__ velS) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int c = sortedHash[k];
    int s = __ldg(cellOffset + c), e = __ldg(cellOffset + c + 1);
    int my = tmpIds[k];
    int r = 0;
    for (int t = s; t < e; t++) r += __ldg(tmpIds + t) < my;
    int dst = s + r;
    sortedIds[dst] = my;
    posS[dst] = __ldg(pos + my);
    velS[dst] = __ldg(vel + my);
}

void launch_rank_gather(int n, SortBuffers sb, const float4* pos, const float4* vel, float4* posS,
                        float4* velS, cudaStream_t s) {
    if (n <= 0) return;
    k_rank_gather<<<(n + 255) / 256, 256, 0, s>>>(n, sb.sortedHash, sb.cellOffset, sb.tmpIds, pos, vel,
                                                  sb.sortedIds, posS, velS);
}

// ---------------------------------------------------------------------------
// Neighbour rows: the 3x3 (z, y) rows of the 27-cell stencil.  Cells of one
// row are consecutive hashes, so the candidates of a row are one contiguous
// range of the sorted arrays, visited in the reference's k, j, i order.
// ---------------------------------------------------------------------------
struct Stencil {
    int x0, x1, y0, y1, z0, z1;
};

__device__ __forceinline__ Stencil stencil(float4 x, float h, const GridDev& g) {
    Stencil s;
    s.x0 = grid_coord(x.x, -h, g.origin[0], g.spacing, g.dim[0]);
    s.x1 = grid_coord(x.x, h, g.origin[0], g.spacing, g.dim[0]);
    s.y0 = grid_coord(x.y, -h, g.origin[1], g.spacing, g.dim[1]);
    s.y1 = grid_coord(x.y, h, g.origin[1], g.spacing, g.dim[1]);
    s.z0 = grid_coord(x.z, -h, g.origin[2], g.spacing, g.dim[2]);
    s.z1 = grid_coord(x.z, h, g.origin[2], g.spacing, g.dim[2]);
    return s;
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float term) {
    float y = __fsub_rn(term, comp);
    float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

// ---------------------------------------------------------------------------
// Stage 5: density + pressure (compute_particle_density_pressure,
// particle_simulation.cu:196-256).  Branch-free poly6 accumulation.
// Writes (rho, p, p/rho^2, 1/rho) for the force stage.
// ---------------------------------------------------------------------------
template <bool KAHAN, bool MAP>
__global__ void __launch_bounds__(256)
k_density(int n, const float4* __restrict__ posS, const int* __restrict__ cellOffset, GridDev g,
          PhysDev ph, MapDev map, float4* __restrict__ rho4S) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = posS[i];
    const Stencil st = stencil(xi, ph.h, g);
    float sum = 0.f, comp = 0.f;
    for (int z = st.z0; z <= st.z1; z++) {
        for (int y = st.y0; y <= st.y1; y++) {
            const int row = g.dim[0] * (g.dim[1] * z + y);
            const int s = __ldg(cellOffset + row + st.x0);
            const int e = __ldg(cellOffset + row + st.x1 + 1);
            for (int t = s; t < e; t++) {
                const float4 xj = __ldg(posS + t);
                const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float w = fmaxf(ph.h2 - r2, 0.f);
                const float term = w * w * w;
                if (KAHAN) kahan_add(sum, comp, term);
                else sum += term;
            }
        }
    }
    float rho = (KAHAN ? __fsub_rn(sum, comp) : sum) * ph.poly6m;
    if (MAP) {
        float uvw[3];
        map_uvw(map, xi, uvw);
        rho += tri_vec(map, uvw[0], uvw[1], uvw[2]).y;
    }
    const float p = ph.stiffness * (rho - ph.restDensity);
    const float inv = 1.0f / rho;
    rho4S[i] = make_float4(rho, p, p * inv * inv, inv);
}

void launch_density(int n, const float4* posS, const int* cellOffset, GridDev g, PhysDev ph,
                    MapDev map, float4* rho4S, int kahan, int blockSize, cudaStream_t s) {
    if (n <= 0) return;
    int bs = blockSize > 0 ? blockSize : 128;
    int grid = (n + bs - 1) / bs;
    if (kahan) {
        if (map.present) k_density<true, true><<<grid, bs, 0, s>>>(n, posS, cellOffset, g, ph, map, rho4S);
        else k_density<true, false><<<grid, bs, 0, s>>>(n, posS, cellOffset, g, ph, map, rho4S);
    } else {
        if (map.present) k_density<false, true><<<grid, bs, 0, s>>>(n, posS, cellOffset, g, ph, map, rho4S);
        else k_density<false, false><<<grid, bs, 0, s>>>(n, posS, cellOffset, g, ph, map, rho4S);
    }
}

// ---------------------------------------------------------------------------
// Stage 6: forces + wall terms + integration + box collision
// (compute_particle_acceleration_ifsurf :315-474, integrate_euler :632-665,
//  collision_handling :742-834), then the new state is written back in
// particle-index order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void collide(const PhysDev& ph, float3& x, float3& v) {
    float lx = x.x - ph.boxCen[0], ly = x.y - ph.boxCen[1], lz = x.z - ph.boxCen[2];
    float dist = fmaxf(fmaxf(fabsf(lx) - ph.boxDim[0], fabsf(ly) - ph.boxDim[1]),
                       fabsf(lz) - ph.boxDim[2]);
    if (!(dist > 0.f)) return;
    float cx = fminf(ph.boxDim[0], fmaxf(-ph.boxDim[0], lx)) + ph.boxCen[0];
    float cy = fminf(ph.boxDim[1], fmaxf(-ph.boxDim[1], ly)) + ph.boxCen[1];
    float cz = fminf(ph.boxDim[2], fmaxf(-ph.boxDim[2], lz)) + ph.boxCen[2];
    float nx = x.x - cx, ny = x.y - cy, nz = x.z - cz;
    float depth = sqrtf(nx * nx + ny * ny + nz * nz);
    if (!(depth > 0.f)) return;
    nx /= depth;
    ny /= depth;
    nz /= depth;
    float velNorm = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    float dp = nx * v.x + ny * v.y + nz * v.z;
    float coeff = velNorm > 0.f ? (1.f + ph.restitution * depth / (ph.dtCollide * velNorm)) * dp : dp;
    v.x -= coeff * nx;
    v.y -= coeff * ny;
    v.z -= coeff * nz;
    x = make_float3(cx, cy, cz);
}

template <bool KAHAN, bool MAP, bool TENSION, bool COLLIDE>
__global__ void __launch_bounds__(256)
k_force(int n, const float4* __restrict__ posS, const float4* __restrict__ velS,
        const float4* __restrict__ rho4S, const int* __restrict__ sortedIds,
        const int* __restrict__ cellOffset, GridDev g, PhysDev ph, MapDev map,
        float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ accS) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = posS[i];
    const float4 vi = velS[i];
    const float4 ri = rho4S[i];
    const Stencil st = stencil(xi, ph.h, g);
    float fp[3] = {0.f, 0.f, 0.f}, cp[3] = {0.f, 0.f, 0.f};
    float fv[3] = {0.f, 0.f, 0.f}, cv[3] = {0.f, 0.f, 0.f};
    float cg[3] = {0.f, 0.f, 0.f}, cl = 0.f;
    for (int z = st.z0; z <= st.z1; z++) {
        for (int y = st.y0; y <= st.y1; y++) {
            const int row = g.dim[0] * (g.dim[1] * z + y);
            const int s = __ldg(cellOffset + row + st.x0);
            const int e = __ldg(cellOffset + row + st.x1 + 1);
            for (int t = s; t < e; t++) {
                const float4 xj = __ldg(posS + t);
                const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 <= ph.h2 && r2 > 0.f) {
                    const float rinv = rsqrtf(r2);
                    const float hr = ph.h - r2 * rinv;
                    const float4 rj = __ldg(rho4S + t);
                    const float4 vj = __ldg(velS + t);
                    const float sp = (ri.z + rj.z) * hr * hr * rinv;
                    const float sv = rj.w * hr;
                    const float tp[3] = {sp * dx, sp * dy, sp * dz};
                    const float tv[3] = {sv * (vj.x - vi.x), sv * (vj.y - vi.y), sv * (vj.z - vi.z)};
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        if (KAHAN) {
                            kahan_add(fp[a], cp[a], tp[a]);
                            kahan_add(fv[a], cv[a], tv[a]);
                        } else {
                            fp[a] += tp[a];
                            fv[a] += tv[a];
                        }
                    }
                    if (TENSION) {
                        const float d2 = ph.h2 - r2;
                        const float sc = rj.w * d2 * d2;
                        cg[0] += sc * dx;
                        cg[1] += sc * dy;
                        cg[2] += sc * dz;
                        cl += rj.w * d2 * (3.f * ph.h2 - 7.f * r2);
                    }
                }
            }
        }
    }
    const float rho = ri.x;
    const float pc = ph.pressCoef * rho;
    float force[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float P = KAHAN ? __fsub_rn(fp[a], cp[a]) : fp[a];
        float V = KAHAN ? __fsub_rn(fv[a], cv[a]) : fv[a];
        force[a] = ph.viscCoef * V + pc * P;
    }
    bool tension = TENSION;
    if (MAP) {
        float uvw[3];
        map_uvw(map, xi, uvw);
        const float4 s = tri_vec(map, uvw[0], uvw[1], uvw[2]);
        const float distWall = -s.x;
        if (distWall < map.restDistance) {
            tension = false;
            const float coeff = rho / (ph.dtCollide * ph.dtCollide) * (map.restDistance - distWall);
            float gN[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                float up[3] = {uvw[0], uvw[1], uvw[2]}, dn[3] = {uvw[0], uvw[1], uvw[2]};
                up[a] = uvw[a] + map.du[a];
                dn[a] = uvw[a] - map.du[a];
                gN[a] = (tri_scalar(map, map.dist, up[0], up[1], up[2]) -
                         tri_scalar(map, map.dist, dn[0], dn[1], dn[2])) / (2.f * map.du[a]);
            }
            force[0] -= coeff * gN[0] + vi.x * s.z;
            force[1] -= coeff * gN[1] + vi.y * s.z;
            force[2] -= coeff * gN[2] + vi.z * s.z;
        }
    }
    if (TENSION && tension) {
        const float cgx = ph.cgCoef * cg[0], cgy = ph.cgCoef * cg[1], cgz = ph.cgCoef * cg[2];
        const float norm = sqrtf(cgx * cgx + cgy * cgy + cgz * cgz);
        if (norm > ph.normThresh) {
            const float fc = ph.tension * (ph.clCoef * cl) / norm;
            force[0] -= fc * cgx;
            force[1] -= fc * cgy;
            force[2] -= fc * cgz;
        }
    }
    float acc[3] = {force[0] / rho, force[1] / rho, force[2] / rho};
    acc[0] -= ph.gravityAxis == 0 ? ph.gravity : 0.f;
    acc[1] -= ph.gravityAxis == 1 ? ph.gravity : 0.f;
    acc[2] -= ph.gravityAxis == 2 ? ph.gravity : 0.f;
    float3 v = make_float3(vi.x + ph.dt * acc[0], vi.y + ph.dt * acc[1], vi.z + ph.dt * acc[2]);
    float3 x = make_float3(xi.x + ph.dt * v.x, xi.y + ph.dt * v.y, xi.z + ph.dt * v.z);
    if (COLLIDE) collide(ph, x, v);
    const int id = sortedIds[i];
    pos[id] = make_float4(x.x, x.y, x.z, 0.f);
    vel[id] = make_float4(v.x, v.y, v.z, 0.f);
    accS[i] = make_float4(acc[0], acc[1], acc[2], 0.f);
}

template <bool KAHAN, bool MAP, bool TENSION>
static void force_collide(bool collide, int grid, int bs, cudaStream_t s, int n, const float4* posS,
                          const float4* velS, const float4* rho4S, const int* ids, const int* off,
                          GridDev g, PhysDev ph, MapDev map, float4* pos, float4* vel, float4* accS) {
    if (collide)
        k_force<KAHAN, MAP, TENSION, true><<<grid, bs, 0, s>>>(n, posS, velS, rho4S, ids, off, g, ph, map,
                                                               pos, vel, accS);
    else
        k_force<KAHAN, MAP, TENSION, false><<<grid, bs, 0, s>>>(n, posS, velS, rho4S, ids, off, g, ph, map,
                                                                pos, vel, accS);
}

template <bool KAHAN>
static void force_map(bool hasMap, bool tension, bool collide, int grid, int bs, cudaStream_t s, int n,
                      const float4* posS, const float4* velS, const float4* rho4S, const int* ids,
                      const int* off, GridDev g, PhysDev ph, MapDev map, float4* pos, float4* vel,
                      float4* accS) {
    if (hasMap) {
        if (tension) force_collide<KAHAN, true, true>(collide, grid, bs, s, n, posS, velS, rho4S, ids, off, g, ph, map, pos, vel, accS);
        else force_collide<KAHAN, true, false>(collide, grid, bs, s, n, posS, velS, rho4S, ids, off, g, ph, map, pos, vel, accS);
    } else {
        if (tension) force_collide<KAHAN, false, true>(collide, grid, bs, s, n, posS, velS, rho4S, ids, off, g, ph, map, pos, vel, accS);
        else force_collide<KAHAN, false, false>(collide, grid, bs, s, n, posS, velS, rho4S, ids, off, g, ph, map, pos, vel, accS);
    }
}

void launch_force(int n, const float4* posS, const float4* velS, const float4* rho4S,
                  const int* sortedIds, const int* cellOffset, GridDev g, PhysDev ph, MapDev map,
                  int collide, float4* pos, float4* vel, float4* accS, int kahan, int blockSize,
                  cudaStream_t s) {
    if (n <= 0) return;
    int bs = blockSize > 0 ? blockSize : 128;
    int grid = (n + bs - 1) / bs;
    bool tension = ph.tension != 0.0f;
    if (kahan)
        force_map<true>(map.present != 0, tension, collide != 0, grid, bs, s, n, posS, velS, rho4S, sortedIds,
                        cellOffset, g, ph, map, pos, vel, accS);
    else
        force_map<false>(map.present != 0, tension, collide != 0, grid, bs, s, n, posS, velS, rho4S,
                         sortedIds, cellOffset, g, ph, map, pos, vel, accS);
}

// ---------------------------------------------------------------------------
// Read-back helpers
// ---------------------------------------------------------------------------
__global__ void k_unpermute(int n, const int* __restrict__ ids, const float4* __restrict__ src, int comp,
                            float* __restrict__ dst, int stride, int offset) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float4 v = src[k];
    float* o = dst + (size_t)ids[k] * stride + offset;
    if (comp < 0) {
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
    } else {
        o[0] = comp == 0 ? v.x : comp == 1 ? v.y : comp == 2 ? v.z : v.w;
    }
}

void launch_unpermute(int n, const int* sortedIds, const float4* srcS, int comp, float* dst, int stride,
                      int offset, cudaStream_t s) {
    if (n <= 0) return;
    k_unpermute<<<(n + 255) / 256, 256, 0, s>>>(n, sortedIds, srcS, comp, dst, stride, offset);
}

// Reference cell tables from the offsets: EMPTY (0xFFFFFFFF) for empty cells.
__global__ void k_cell_tables(int numCells, const int* __restrict__ off, int* start, int* end) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCells) return;
    int s = off[c], e = off[c + 1];
    bool occ = e > s;
    if (start) start[c] = occ ? s : -1;
    if (end) end[c] = occ ? e : -1;
}

void launch_cell_tables(int numCells, const int* cellOffset, int* start, int* end, cudaStream_t s) {
    if (numCells <= 0) return;
    k_cell_tables<<<(numCells + 255) / 256, 256, 0, s>>>(numCells, cellOffset, start, end);
}

}  // namespace sph
