// Sorting stages of the GB300 SPH step and read-back helpers.
//
// Data layout in HBM (one handle, n particles, C cells):
//   pos, vel           float4[n]  particle-index order (the state; pos.w: the
//                                 scene of a batched handle, or the packed cell of
//                                 a cell-relative one)
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

#include <algorithm>
#include <cstdlib>

#include "sph_device.cuh"

namespace sph {

// ---------------------------------------------------------------------------
// AoS <-> float4 conversion (VD/SD layouts of particle_simulation.h:17-41)
// ---------------------------------------------------------------------------
__global__ void k_set_scene(float4* __restrict__ pos, int count, int sid) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) pos[i].w = __int_as_float(sid);
}

void launch_set_scene(float4* pos, int count, int sid, cudaStream_t s) {
    if (count > 0) k_set_scene<<<(count + 255) / 256, 256, 0, s>>>(pos, count, sid);
}

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

// Cell-relative state <-> absolute positions (sph_options.cellRelative).
__global__ void k_abs_to_rel(int n, float4* __restrict__ pos, GridDev g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    float3 rel;
    int3 c;
    rel_from_abs(make_float3(p.x, p.y, p.z), g, rel, c);
    pos[i] = make_float4(rel.x, rel.y, rel.z, rel_pack(c.x, c.y, c.z));
}

__global__ void k_rel_to_abs(int n, const float4* __restrict__ in, GridDev g, float* __restrict__ aos, int stride,
                             float4* __restrict__ out4) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = in[i];
    const float4 a = rel_abs(p, rel_cell(p), g);
    if (aos) {
        float* p = aos + (size_t)i * stride;
        p[0] = a.x;
        p[1] = a.y;
        p[2] = a.z;
    }
    if (out4) out4[i] = make_float4(a.x, a.y, a.z, 0.f);
}

void launch_abs_to_rel(int n, float4* pos, GridDev g, cudaStream_t s) {
    if (n > 0) k_abs_to_rel<<<(n + 255) / 256, 256, 0, s>>>(n, pos, g);
}

void launch_rel_to_abs(int n, const float4* pos, GridDev g, float* aos, int stride, float4* out4, cudaStream_t s) {
    if (n > 0) k_rel_to_abs<<<(n + 255) / 256, 256, 0, s>>>(n, pos, g, aos, stride, out4);
}

void launch_unpack_aos(const float* aos, int stride, int offset, int n, float4* out, cudaStream_t s) {
    if (n <= 0) return;
    k_unpack_aos<<<(n + 255) / 256, 256, 0, s>>>(aos, stride, offset, n, out);
}

// VD / velocity layout (three floats per particle) into a 16-byte aligned
// destination: each block stages its 256 particles' 768 floats in shared
// memory and stores them as 16-byte vectors, the trailing 0-3 floats singly.
// Into page-locked host memory this runs at the host link's rate (12 MB in
// ~68 us on GB300), where single-float stores and a pack followed by a DMA
// copy take ~80 us.
__global__ void __launch_bounds__(256) k_pack3_vec(const float4* __restrict__ in, int n, float* __restrict__ aos) {
    __shared__ __align__(16) float sm[768];
    const int base = blockIdx.x * 256;
    const int cnt = min(256, n - base);
    const int nf = cnt * 3, nv = nf >> 2;
    const int t = threadIdx.x;
    if (t < cnt) {
        const float4 v = in[base + t];
        sm[3 * t] = v.x;
        sm[3 * t + 1] = v.y;
        sm[3 * t + 2] = v.z;
    }
    __syncthreads();
    float* dst = aos + (size_t)base * 3;  // 3072-byte steps from an aligned start
    for (int k = t; k < nv; k += 256) reinterpret_cast<float4*>(dst)[k] = reinterpret_cast<const float4*>(sm)[k];
    for (int k = nv * 4 + t; k < nf; k += 256) dst[k] = sm[k];
}

void launch_pack_aos(const float4* in, int n, float* aos, int stride, int offset, cudaStream_t s) {
    if (n <= 0) return;
    if (stride == 3 && offset == 0 && (reinterpret_cast<uintptr_t>(aos) & 15) == 0)
        k_pack3_vec<<<(n + 255) / 256, 256, 0, s>>>(in, n, aos);
    else
        k_pack_aos<<<(n + 255) / 256, 256, 0, s>>>(in, n, aos, stride, offset);
}

// ---------------------------------------------------------------------------
// Stage 1: hash + per-cell arrival slot
// ---------------------------------------------------------------------------
// With BATCH the particle's scene (pos.w) supplies its grid, whose cells
// start at that scene's cellBase in the concatenated cell space.
// With REL the position is cell-relative and the hash comes from its packed
// cell coordinates.
// With reused neighbour lists the pass returns at once in a step that builds
// none (k_list_decide has decided; the rank pass checks the state instead).
template <bool BATCH, bool REL>
__global__ void k_hash_count(int n, const float4* __restrict__ pos, GridDev g_, const SceneDev* __restrict__ scenes,
                             int* __restrict__ cnt, int2* __restrict__ keySlot, unsigned int* status,
                             const int* __restrict__ skip, const unsigned int* __restrict__ sortFlag) {
    if ((sortFlag && !*sortFlag) || (skip && *skip)) return;
    // one wave of blocks striding over the particles (a step that returns
    // at once then costs one wave; the arrival order in a cell is ranked
    // away later, so the grid shape changes no result)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = pos[i];
        const GridDev& g = BATCH ? scenes[__float_as_int(p.w)].g : g_;
        bool outside = false;
        const bool finite = isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
        if (!finite) {
            atomicOr(status, STATUS_NON_FINITE);
            p = make_float4(g.origin[0], g.origin[1], g.origin[2], 0.f);
        }
        int h;
        if (REL) {
            const int3 c = finite ? rel_cell(p) : make_int3(0, 0, 0);
            h = g.cellBase + g.dim[0] * (g.dim[1] * c.z + c.y) + c.x;
        } else {
            h = particle_hash(p, g, &outside);
        }
        if (outside) atomicOr(status, STATUS_OUT_OF_DOMAIN);
        int slot = atomicAdd(cnt + h, 1);
        keySlot[i] = make_int2(h, slot);
    }
}

// Blocks of 256 threads for the striding sort passes: one full wave.
static int stride_blocks(int n) {
    const int want = (n + 255) / 256;
    return std::max(1, std::min(want, device_sms() * (2048 / 256)));
}

// Reused neighbour lists: whether each scene builds them in this step (on
// request, or when one of its particles has moved farther than the skin
// allows since the last build, or the displacement is not finite; thread k
// decides scene k), whether the step sorts (some scene builds) and whether
// it leaves the cell tables stale (it does not sort).  One block.
__global__ void k_list_decide(NeighbourLists L, const SceneDev* __restrict__ scenes) {
    __shared__ int anyBuild;
    if (threadIdx.x == 0) anyBuild = 0;
    __syncthreads();
    const int S = L.numScenes;
    unsigned int* f = L.flags;
    for (int k = threadIdx.x; k < S; k += blockDim.x) {
        float lim2 = L.dispLimit2;
        if (scenes) {
            const float lim = 0.45f * L.skinFrac * scenes[k].ph.h;
            lim2 = lim * lim;
        }
        const float d2 = __uint_as_float(f[VL_DISP * S + k]);
        const bool build = f[VL_BUILD * S + k] != 0u || !(d2 <= lim2);
        f[VL_BUILD_NOW * S + k] = build ? 1u : 0u;
        f[VL_BUILD * S + k] = 0u;
        if (build) {
            f[VL_DISP * S + k] = 0u;
            f[VL_COUNT * S + k] += 1u;
            anyBuild = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        f[VL_FLAGS * S + VL_SORT] = anyBuild ? 1u : 0u;
        f[VL_FLAGS * S + VL_STALE] = anyBuild ? 0u : 1u;
    }
}

static const unsigned int* sort_flag(const NeighbourLists* L) {
    return L ? L->flags + VL_FLAGS * L->numScenes + VL_SORT : nullptr;
}

void launch_hash_count(int n, const float4* pos, GridDev g, SortBuffers sb, unsigned int* status,
                       cudaStream_t s, const NeighbourLists* L) {
    if (n <= 0) return;
    if (L) k_list_decide<<<1, 256, 0, s>>>(*L, sb.scenes);
    const unsigned int* sf = sort_flag(L);
    const int grid = stride_blocks(n);
    if (sb.scenes)
        k_hash_count<true, false><<<grid, 256, 0, s>>>(n, pos, g, sb.scenes, sb.cnt, sb.keySlot, status, sb.skip, sf);
    else if (g.rel)
        k_hash_count<false, true><<<grid, 256, 0, s>>>(n, pos, g, nullptr, sb.cnt, sb.keySlot, status, sb.skip,
                                                       nullptr);
    else
        k_hash_count<false, false><<<grid, 256, 0, s>>>(n, pos, g, nullptr, sb.cnt, sb.keySlot, status, sb.skip, sf);
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

// `waitLimit` bounds each spin (polls); a negative limit abandons every wait
// at its first poll (a test of the give-up path: every tile then takes its
// predecessors as zero).  A tile that gives up latches STATUS_DEVICE_WAIT and
// completes with a prefix that is a partial sum of the true one, so every
// offset stays within [0, n] and every index derived from the offsets stays
// inside its buffer (the step's results are then unspecified and reported).
__global__ void __launch_bounds__(SCAN_THREADS)
k_cell_scan(int total, int* __restrict__ cnt, int* __restrict__ out, unsigned long long* flags,
            unsigned int* tileCounter, unsigned int* status, const int* __restrict__ skip, int waitLimit,
            const unsigned int* __restrict__ sortFlag) {
    // every block alike: no tile is taken, none waited on
    if ((skip && *skip) || (sortFlag && !*sortFlag)) return;
    __shared__ int s_tile;
    __shared__ int s_warp[SCAN_THREADS / 32];
    __shared__ int s_prefix;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(tileCounter, 1u);
    __syncthreads();
    const int tile = s_tile;
    const int base = tile * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    static_assert(SCAN_ITEMS % 4 == 0, "vector loads of four counters");
    if (base + SCAN_ITEMS <= total) {
#pragma unroll
        for (int c = 0; c < SCAN_ITEMS / 4; c++) {
            const int4 a = *reinterpret_cast<const int4*>(cnt + base + 4 * c);
            v[4 * c] = a.x;
            v[4 * c + 1] = a.y;
            v[4 * c + 2] = a.z;
            v[4 * c + 3] = a.w;
            *reinterpret_cast<int4*>(cnt + base + 4 * c) = make_int4(0, 0, 0, 0);
        }
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
                    if (waitLimit < 0) {
                        atomicOr(status, STATUS_DEVICE_WAIT);
                        f = FLAG_INC;  // the wait abandoned at once
                    }
                    while ((f >> 32) == 0ull) {
                        if (++spins > waitLimit) {
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
#pragma unroll
        for (int c = 0; c < SCAN_ITEMS / 4; c++) {
            int4 o;
            o.x = run;
            run += v[4 * c];
            o.y = run;
            run += v[4 * c + 1];
            o.z = run;
            run += v[4 * c + 2];
            o.w = run;
            run += v[4 * c + 3];
            *reinterpret_cast<int4*>(out + base + 4 * c) = o;
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            if (base + k < total) out[base + k] = run;
            run += v[k];
        }
    }
}

// The look-back's poll limit: SPIN_LIMIT, or the integer in the environment
// variable SPH_SCAN_WAIT_LIMIT (read at each launch; a captured step graph
// keeps the value it was captured with).  Tests set it to exercise the
// give-up path; -1 abandons every wait at once.
static int scan_wait_limit() {
    const char* e = getenv("SPH_SCAN_WAIT_LIMIT");
    if (!e || !*e) return SPIN_LIMIT;
    return (int)strtol(e, nullptr, 10);
}

void launch_cell_scan(int numCells, SortBuffers sb, unsigned int* status, cudaStream_t s, const NeighbourLists* L) {
    int total = numCells + 1;
    int tiles = (total + SCAN_TILE - 1) / SCAN_TILE;
    // tile counter (first 16 bytes) and the tile states that follow it
    cudaMemsetAsync(sb.tileCounter, 0, 16 + sizeof(unsigned long long) * (size_t)tiles, s);
    k_cell_scan<<<tiles, SCAN_THREADS, 0, s>>>(total, sb.cnt, sb.cellOffset, sb.scanFlags,
                                               sb.tileCounter, status, sb.skip, scan_wait_limit(), sort_flag(L));
}

// ---------------------------------------------------------------------------
// Stage 3: scatter ids into their cell segments (arrival order)
// ---------------------------------------------------------------------------
// After a scan wait gave up (status) the scatter and the rank pass leave
// their outputs as they were: the step's results are unspecified and the
// condition is reported.
__global__ void k_scatter(int n, const int2* __restrict__ keySlot, const int* __restrict__ cellOffset,
                          int* __restrict__ tmpIds, int* __restrict__ sortedHash, const int* __restrict__ skip,
                          const unsigned int* __restrict__ status, const unsigned int* __restrict__ sortFlag) {
    if ((skip && *skip) || (status && (*status & STATUS_DEVICE_WAIT)) || (sortFlag && !*sortFlag)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int2 ks = keySlot[i];
        int dst = __ldg(cellOffset + ks.x) + ks.y;
        tmpIds[dst] = i;
        sortedHash[dst] = ks.x;
    }
}

void launch_scatter(int n, SortBuffers sb, cudaStream_t s, const unsigned int* status, const NeighbourLists* L) {
    if (n <= 0) return;
    k_scatter<<<stride_blocks(n), 256, 0, s>>>(n, sb.keySlot, sb.cellOffset, sb.tmpIds, sb.sortedHash, sb.skip,
                                               status, sort_flag(L));
}

// ---------------------------------------------------------------------------
// Stage 4: order each cell's members and gather the state into sorted order.
// Two orders come out of one pass over the cell segment:
//   by particle id   -> sortedIds, the reference's permutation (stable sort
//                       by hash, particle_simulation.cu:2340), kept for the API;
//   by (x, id)       -> workIds, the order the neighbour kernels use: a cell's
//                       members sorted by x, so the lower and upper x-halves of
//                       a cell are two contiguous ranges (halfOffset below).
// Ranks count the smaller keys in the segment; x is compared through its
// order-preserving integer image so the order is total (NaN included).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned int ordered_bits(float x) {
    unsigned int u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// The same pass records, per cell, where its upper x-half starts in the
// working order (halfOffset[c] = first index with x >= the cell's mid-plane),
// so a neighbour search can cut a row at half-cell granularity from a table.
// With reused neighbour lists (`vl`) and no build in this step, the working
// order is the one kept since the build (workIds): only the reference
// permutation is ranked, and the state is gathered into the kept order.
template <bool BATCH, bool REL>
__global__ void k_rank_gather(int n, const int* __restrict__ sortedHash, const int* __restrict__ cellOffset,
                              const int* __restrict__ tmpIds, const float4* __restrict__ pos,
                              const float4* __restrict__ vel, GridDev g_, const SceneDev* __restrict__ scenes,
                              int* __restrict__ sortedIds, int* __restrict__ workIds, int* __restrict__ halfOffset,
                              float4* __restrict__ posS, float4* __restrict__ velS, const int* __restrict__ skip,
                              const unsigned int* __restrict__ vl, int vlScenes, const int* __restrict__ slotScene,
                              unsigned int* status) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || (skip && *skip) || (status && (*status & STATUS_DEVICE_WAIT))) return;
    const int sc = BATCH && vl ? slotScene[k] : 0;  // the scene of sorted slot k
    if (vl && !vl[VL_FLAGS * vlScenes + VL_SORT]) {
        // no sort in this step: the state gathered into the kept order, with
        // the hash pass's checks of each position
        const int w = workIds[k];
        const float4 p = __ldg(pos + w);
        posS[k] = p;
        velS[k] = __ldg(vel + w);
        const GridDev& g = BATCH ? scenes[sc].g : g_;
        if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) {
            atomicOr(status, STATUS_NON_FINITE);
        } else {
            bool outside = false;
            particle_hash(p, g, &outside);
            if (outside) atomicOr(status, STATUS_OUT_OF_DOMAIN);
        }
        return;
    }
    int c = sortedHash[k];
    int s = __ldg(cellOffset + c), e = __ldg(cellOffset + c + 1);
    int my = tmpIds[k];
    if (vl && !vl[VL_BUILD_NOW * vlScenes + sc]) {
        int rId = 0;
        for (int t = s; t < e; t++) rId += __ldg(tmpIds + t) < my;
        sortedIds[s + rId] = my;
        const int w = workIds[k];
        posS[k] = __ldg(pos + w);
        velS[k] = __ldg(vel + w);
        return;
    }
    float4 p = __ldg(pos + my);
    const GridDev& g = BATCH ? scenes[__float_as_int(p.w)].g : g_;
    unsigned int key = ordered_bits(p.x);
    // the cell's mid-plane, in the frame its members' x is stored in
    const float mid = REL ? 0.5f * g.spacing
                          : g.origin[0] + ((float)((c - g.cellBase) % g.dim[0]) + 0.5f) * g.spacing;
    int rId = 0, rX = 0, below = 0;
    for (int t = s; t < e; t++) {
        int o = __ldg(tmpIds + t);
        float xo = __ldg(&pos[o].x);
        unsigned int ko = ordered_bits(xo);
        rId += o < my;
        rX += (ko < key) || (ko == key && o < my);
        below += xo < mid;
    }
    sortedIds[s + rId] = my;
    workIds[s + rX] = my;
    posS[s + rX] = p;
    velS[s + rX] = __ldg(vel + my);
    if (rX == 0) halfOffset[c] = s + below;
}

void launch_rank_gather(int n, SortBuffers sb, const float4* pos, const float4* vel, GridDev g, float4* posS,
                        float4* velS, cudaStream_t s, const NeighbourLists* L, unsigned int* status) {
    if (n <= 0) return;
    const int grid = (n + 255) / 256;
    const unsigned int* vl = L ? L->flags : nullptr;
    const int vs = L ? L->numScenes : 1;
    const int* ss = L ? L->slotScene : nullptr;
    if (sb.scenes)
        k_rank_gather<true, false><<<grid, 256, 0, s>>>(n, sb.sortedHash, sb.cellOffset, sb.tmpIds, pos, vel, g,
                                                        sb.scenes, sb.sortedIds, sb.workIds, sb.halfOffset, posS,
                                                        velS, sb.skip, vl, vs, ss, status);
    else if (g.rel)
        k_rank_gather<false, true><<<grid, 256, 0, s>>>(n, sb.sortedHash, sb.cellOffset, sb.tmpIds, pos, vel, g,
                                                        nullptr, sb.sortedIds, sb.workIds, sb.halfOffset, posS, velS,
                                                        sb.skip, nullptr, 1, nullptr, status);
    else
        k_rank_gather<false, false><<<grid, 256, 0, s>>>(n, sb.sortedHash, sb.cellOffset, sb.tmpIds, pos, vel, g,
                                                         nullptr, sb.sortedIds, sb.workIds, sb.halfOffset, posS,
                                                         velS, sb.skip, vl, vs, nullptr, status);
}

// ---------------------------------------------------------------------------
// Cell tables after a step that skipped them (reused lists, no build): the
// step's positions are those of its sorted copies (in the kept working
// order), so the tables are rebuilt from them -- the hash, scan and scatter
// over the positions put back in particle order, then the rank by id within
// each cell -- exactly as the step would have built them.
// ---------------------------------------------------------------------------
__global__ void k_unsort_positions(int n, const float4* __restrict__ posS, const int* __restrict__ workIds,
                                   const int* __restrict__ slotScene, float4* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 p = posS[k];  // (its fourth lane holds p/rho^2: the scene, for a batch, from the slot)
    out[workIds[k]] = make_float4(p.x, p.y, p.z, slotScene ? __int_as_float(slotScene[k]) : 0.f);
}

__global__ void k_rank_ids(int n, const int* __restrict__ sortedHash, const int* __restrict__ cellOffset,
                           const int* __restrict__ tmpIds, int* __restrict__ sortedIds) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int c = sortedHash[k];
    const int s = __ldg(cellOffset + c), e = __ldg(cellOffset + c + 1);
    const int my = tmpIds[k];
    int rId = 0;
    for (int t = s; t < e; t++) rId += __ldg(tmpIds + t) < my;
    sortedIds[s + rId] = my;
}

void launch_rebuild_tables(int n, const float4* posS, const int* workIds, const int* slotScene, GridDev g,
                           SortBuffers sb, float4* scratch, unsigned int* status, cudaStream_t s) {
    if (n <= 0) return;
    sb.skip = nullptr;
    k_unsort_positions<<<(n + 255) / 256, 256, 0, s>>>(n, posS, workIds, slotScene, scratch);
    launch_hash_count(n, scratch, g, sb, status, s, nullptr);
    launch_cell_scan(g.numCells, sb, status, s, nullptr);
    launch_scatter(n, sb, s, status, nullptr);
    k_rank_ids<<<(n + 255) / 256, 256, 0, s>>>(n, sb.sortedHash, sb.cellOffset, sb.tmpIds, sb.sortedIds);
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
