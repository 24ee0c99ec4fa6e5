// The two-scale pass (AdvanceTwoScale, particle_simulation.cu:2145-2182, and
// AdvanceSubParticles, :2119-2143) on the GPU.
//
// Every coarse particle keeps a 2-bit state history (split / boundary /
// default); split and boundary particles get 8 children each, in persistent
// slots 8*parent + k of the child arrays.  Children of split particles
// ("regular") get densities and forces at h/2 on the fine grid; children of
// boundary particles get the mean coarse density and pressure around them.
// All children are integrated and collided.  With childMode 0 children are
// re-seeded in every step and nothing feeds back into the coarse particles,
// as in the reference; with childMode 1 they persist while their parent keeps
// its class, and a parent leaving the split class takes its children's mean
// position and velocity (merge-back).
//
// Counts stay on the device: the kernels of the fine level loop over the
// device-side counts (grid-stride), so a two-scale step needs no host
// synchronisation.
#include <cuda/atomic>

#include "sph_device.cuh"

namespace sph {

namespace {

__device__ __forceinline__ bool in_region(const TwoScaleDev& T, float4 x) {
    return x.x >= T.splitMin[0] && x.x <= T.splitMax[0] && x.y >= T.splitMin[1] && x.y <= T.splitMax[1] &&
           x.z >= T.splitMin[2] && x.z <= T.splitMax[2];
}

// r^2 as find_boundary_particles and project_quantities_cell form it
// (:1002-1005, 1317-1321): three products summed left to right, each rounded.
__device__ __forceinline__ float ref_r2(float4 a, float4 b) {
    const float rx = __fsub_rn(a.x, b.x), ry = __fsub_rn(a.y, b.y), rz = __fsub_rn(a.z, b.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz));
}

// Class of a 2-bit state: 1 split (bit 0, as collect reads it), 2 boundary, 0 default.
__device__ __forceinline__ int state_class(unsigned int c) { return (c & 1u) ? 1 : (c == 2u ? 2 : 0); }

inline int stride_grid(long long work, int bs) {
    long long g = (work + bs - 1) / bs;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

// The marking runs over a few thousand split parents, so each gets a warp:
// lane l < 27 takes row l / 3 of the particle's 3 x 3 stencil rows and every
// third candidate of it, from the row's start + l % 3, and loads TS_BATCH
// candidates before it tests any; lanes 27..31 take none.  So a particle
// waits for one round of row offsets and a few rounds of candidate loads,
// not for its rows one after the other.
constexpr int TS_BATCH = 4;
constexpr int TS_WARP_BLOCK = 128;

// stencil() with its six bounds computed by lanes 0..5 (lane 2a + 1 the high
// bound of axis a) and handed to the whole warp; the same values, at a sixth
// of the warp's instructions.
__device__ __forceinline__ Stencil warp_stencil(float4 x, float h, const GridDev& g, int lane) {
    int c = 0;
    if (lane < 6) {
        const int ax = lane >> 1;
        const float p = ax == 0 ? x.x : (ax == 1 ? x.y : x.z);
        const float o = ax == 0 ? g.origin[0] : (ax == 1 ? g.origin[1] : g.origin[2]);
        const int d = ax == 0 ? g.dim[0] : (ax == 1 ? g.dim[1] : g.dim[2]);
        c = grid_coord(p, (lane & 1) ? h : -h, o, g.spacing, d);
    }
    Stencil s;
    s.x0 = __shfl_sync(0xffffffffu, c, 0);
    s.x1 = __shfl_sync(0xffffffffu, c, 1);
    s.y0 = __shfl_sync(0xffffffffu, c, 2);
    s.y1 = __shfl_sync(0xffffffffu, c, 3);
    s.z0 = __shfl_sync(0xffffffffu, c, 4);
    s.z1 = __shfl_sync(0xffffffffu, c, 5);
    return s;
}

__device__ __forceinline__ void lane_row(const Stencil& st, const GridDev& g, const int* __restrict__ offs, int lane,
                                         int& t, int& e) {
    t = e = 0;
    if (lane >= 27) return;
    const int r = lane / 3;
    const int z = st.z0 + r / 3, y = st.y0 + r % 3;
    if (z > st.z1 || y > st.y1) return;
    const int row = g.dim[0] * (g.dim[1] * z + y);
    t = __ldg(offs + row + st.x0) + lane % 3;
    e = __ldg(offs + row + st.x1 + 1);
}

// Calls visit(t, x_t) for the lane's candidates t, with x_t = load(t).
template <class Load, class Visit>
__device__ __forceinline__ void walk_lane(int t, int e, Load load, Visit visit) {
    for (; t < e; t += 3 * TS_BATCH) {
        float4 x[TS_BATCH];
#pragma unroll
        for (int u = 0; u < TS_BATCH; u++)
            if (t + 3 * u < e) x[u] = load(t + 3 * u);
#pragma unroll
        for (int u = 0; u < TS_BATCH; u++)
            if (t + 3 * u < e) visit(t + 3 * u, x[u]);
    }
}

inline int warp_grid(long long items) {
    const long long per = TS_WARP_BLOCK / 32;
    long long b = (items + per - 1) / per;
    const long long cap = 16LL * device_sms();
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// The projection and the fine level's loops run over tens of thousands of
// children: there a particle gets a group of TS_G = 8 lanes (4 per warp), so
// that its setup, stencil and epilogue are shared four ways.  The group
// fetches the bounds of its 9 stencil rows in one round (lane g row g, every
// lane row 8) and walks the rows in order; within a row lane g takes
// candidates start + g, + 8, ... (consecutive lanes read consecutive
// addresses), TS_GBATCH loads in flight.  Group sums use a fixed xor tree
// (every lane of the group ends with the same bits).
constexpr int TS_G = 8;
constexpr int TS_GBATCH = 4;

inline int group_grid(long long items) { return warp_grid((items + 32 / TS_G - 1) / (32 / TS_G)); }

__device__ __forceinline__ Stencil group_stencil(float4 x, float h, const GridDev& g, int gl) {
    int c = 0;
    if (gl < 6) {
        const int ax = gl >> 1;
        const float p = ax == 0 ? x.x : (ax == 1 ? x.y : x.z);
        const float o = ax == 0 ? g.origin[0] : (ax == 1 ? g.origin[1] : g.origin[2]);
        const int d = ax == 0 ? g.dim[0] : (ax == 1 ? g.dim[1] : g.dim[2]);
        c = grid_coord(p, (gl & 1) ? h : -h, o, g.spacing, d);
    }
    Stencil s;
    s.x0 = __shfl_sync(0xffffffffu, c, 0, TS_G);
    s.x1 = __shfl_sync(0xffffffffu, c, 1, TS_G);
    s.y0 = __shfl_sync(0xffffffffu, c, 2, TS_G);
    s.y1 = __shfl_sync(0xffffffffu, c, 3, TS_G);
    s.z0 = __shfl_sync(0xffffffffu, c, 4, TS_G);
    s.z1 = __shfl_sync(0xffffffffu, c, 5, TS_G);
    return s;
}

__device__ __forceinline__ void row_bounds(const Stencil& st, const GridDev& g, const int* __restrict__ offs, int r,
                                           int& s, int& e) {
    s = e = 0;
    const int z = st.z0 + r / 3, y = st.y0 + r % 3;
    if (z > st.z1 || y > st.y1) return;
    const int row = g.dim[0] * (g.dim[1] * z + y);
    s = __ldg(offs + row + st.x0);
    e = __ldg(offs + row + st.x1 + 1);
}

struct GroupRows {
    int s, e;    // row gl
    int s8, e8;  // row 8
};

// All-empty rows for a group without a particle.
__device__ __forceinline__ GroupRows group_rows(const Stencil& st, const GridDev& g, const int* __restrict__ offs,
                                               int gl, bool valid) {
    GroupRows R = {0, 0, 0, 0};
    if (!valid) return R;
    row_bounds(st, g, offs, gl, R.s, R.e);
    row_bounds(st, g, offs, 8, R.s8, R.e8);
    return R;
}

// Bounds of row r (the same in every lane of the group; all lanes call it).
__device__ __forceinline__ void group_row(const GroupRows& R, int r, int& s, int& e) {
    const int a = __shfl_sync(0xffffffffu, R.s, r & 7, TS_G), b = __shfl_sync(0xffffffffu, R.e, r & 7, TS_G);
    s = r < 8 ? a : R.s8;
    e = r < 8 ? b : R.e8;
}

__device__ __forceinline__ float group_total(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
}

// ---------------------------------------------------------------------------
// shift_state + find_split_particles (:730-740, 932-952)
// ---------------------------------------------------------------------------
// Also lists the split particles' working-order indices for the marking
// (warp-aggregated appends, in no fixed order: the marks do not depend on it).
__global__ void k_ts_state(int n, const float4* __restrict__ posS, const int* __restrict__ workIds, TwoScaleDev T) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool split = false;
    if (k < n) {
        const int id = workIds[k];
        unsigned int s = ((unsigned int)T.state[id] << 2) & 0xFFu;
        split = in_region(T, posS[k]);
        if (split) s |= 1u;
        T.state[id] = (unsigned char)s;
    }
    const unsigned int m = __ballot_sync(0xffffffffu, split);
    if (!m) return;
    int base = 0;
    if (lane == 0) base = atomicAdd(T.counts + 4, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (split) T.markList[base + __popc(m & ((1u << lane) - 1u))] = k;
}

// find_boundary_particles (:954-1017) as a race-free scatter: every split
// particle (decided from its position, not from a state other threads are
// changing) marks all particles of its 27-cell stencil within compactSupport,
// itself included, with a word-wide atomic OR.  One warp per listed split
// particle.
__global__ void __launch_bounds__(TS_WARP_BLOCK) k_ts_mark(const float4* __restrict__ posS,
                                                           const int* __restrict__ workIds,
                                                           const int* __restrict__ cellOffset, GridDev g, float h,
                                                           TwoScaleDev T) {
    const int count = T.counts[4];
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (TS_WARP_BLOCK / 32);
    const float h2 = __fmul_rn(h, h);
    unsigned int* words = reinterpret_cast<unsigned int*>(T.state);
    for (int idx = (blockIdx.x * TS_WARP_BLOCK + threadIdx.x) >> 5; idx < count; idx += warps) {
        const float4 xs = posS[T.markList[idx]];
        int t, e;
        lane_row(warp_stencil(xs, h, g, lane), g, cellOffset, lane, t, e);
        walk_lane(t, e, [&](int c) { return __ldg(posS + c); }, [&](int c, float4 xc) {
            if (ref_r2(xs, xc) <= h2) {
                const int v = workIds[c];
                atomicOr(words + (v >> 2), 2u << (8 * (v & 3)));
            }
        });
    }
}

// ---------------------------------------------------------------------------
// collect (:2509-2567): stable three-way compaction in particle order.
// ---------------------------------------------------------------------------
constexpr int TS_BLOCK = 1024;

__device__ __forceinline__ int ts_class(unsigned char s) {
    const int c = s & 3;
    return c == 0 ? 2 : (c == 2 ? 1 : 0);  // 0 split, 1 boundary, 2 default
}

__global__ void __launch_bounds__(TS_BLOCK) k_ts_count(int n, TwoScaleDev T) {
    __shared__ int s_cnt[3];
    if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * TS_BLOCK + threadIdx.x;
    if (i < n) atomicAdd(&s_cnt[ts_class(T.state[i])], 1);
    __syncthreads();
    if (threadIdx.x < 3) T.blockCounts[3 * blockIdx.x + threadIdx.x] = s_cnt[threadIdx.x];
}

// collect_ids (:1118-1162): id lists, and the child list -- split children
// first, then boundary children, 8 consecutive slots per parent.  Each block
// adds up the class counts of the blocks before it (and the split total, the
// boundary children's base) from k_ts_count's table itself, so no separate
// scan launch is needed; the last block writes the totals to the device
// counters.
__global__ void __launch_bounds__(TS_BLOCK) k_ts_lists(int n, TwoScaleDev T) {
    __shared__ int s_warp[3][TS_BLOCK / 32];
    __shared__ int s_red[4][TS_BLOCK / 32];
    __shared__ int s_base[4];  // split, boundary, default before this block; split total
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nb = gridDim.x;
    {
        int v[4] = {0, 0, 0, 0};
        for (int b = threadIdx.x; b < nb; b += TS_BLOCK) {
            const int c0 = T.blockCounts[3 * b], c1 = T.blockCounts[3 * b + 1], c2 = T.blockCounts[3 * b + 2];
            if (b < (int)blockIdx.x) {
                v[0] += c0;
                v[1] += c1;
                v[2] += c2;
            }
            v[3] += c0;
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
            if (lane == 0) s_red[c][warp] = v[c];
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                int w = s_red[c][lane];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
                if (lane == 0) s_base[c] = w;
            }
        }
        __syncthreads();
    }
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) {
        const int tot[3] = {s_base[0] + T.blockCounts[3 * blockIdx.x], s_base[1] + T.blockCounts[3 * blockIdx.x + 1],
                            s_base[2] + T.blockCounts[3 * blockIdx.x + 2]};
        T.counts[0] = tot[0];
        T.counts[1] = tot[1];
        T.counts[2] = tot[2];
        T.counts[3] = 8 * (tot[0] + tot[1]);
        T.counts[4] = 0;  // the marking has read the split list: empty for the next step
    }
    const int i = blockIdx.x * TS_BLOCK + threadIdx.x;
    const int cls = i < n ? ts_class(T.state[i]) : -1;
    int rank[3];
    for (int c = 0; c < 3; c++) {
        const unsigned int m = __ballot_sync(0xffffffffu, cls == c);
        rank[c] = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) s_warp[c][warp] = __popc(m);
    }
    __syncthreads();
    if (warp == 0) {
        for (int c = 0; c < 3; c++) {
            int w = s_warp[c][lane];
            int incl = w;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            s_warp[c][lane] = incl - w;  // exclusive warp offsets
        }
    }
    __syncthreads();
    if (cls < 0) return;
    const int r = s_base[cls] + s_warp[cls][warp] + rank[cls];
    if (cls == 0) {
        T.splitIds[r] = i;
        for (int k = 0; k < 8; k++) T.subIds[8 * r + k] = 8 * i + k;
    } else if (cls == 1) {
        T.boundaryIds[r] = i;
        const int base = 8 * (s_base[3] + r);
        for (int k = 0; k < 8; k++) T.subIds[base + k] = 8 * i + k;
    } else {
        T.defaultIds[r] = i;
    }
}

// compute_sub_particle_hash (:121-153) of the child at list position idx,
// with its arrival slot in its fine cell (the counting sort's first stage).
__device__ __forceinline__ void hash_child(float4 x, const GridDev& sg, const TwoScaleDev& T, int idx,
                                           unsigned int* status) {
    bool outside = false;
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) {
        atomicOr(status, STATUS_NON_FINITE);
        x = make_float4(sg.origin[0], sg.origin[1], sg.origin[2], 0.f);
    }
    const int h = particle_hash(x, sg, &outside);
    if (outside) atomicOr(status, STATUS_OUT_OF_DOMAIN);
    T.subKeySlot[idx] = make_int2(h, atomicAdd(T.subCnt + h, 1));
}

// ---------------------------------------------------------------------------
// initialize_sub_particles (:1023-1090): 8 children on the cube diagonals at
// the radius (3m/(4 pi rho))^(1/3), the parent's velocity.  The radicand is
// formed in double and pow(r, 1.0f/3.0f) evaluated in double and rounded to
// float once; pos + dir*radius is one fused multiply-add, as the reference's
// kernel compiles it.
// ---------------------------------------------------------------------------
//
// Merge-back (childMode 1, no reference counterpart) comes first, in the same
// thread: a parent whose class went from split to boundary or default takes
// the mean of its eight children (summed in slot order, times 1/8) as its
// pre-integration position and velocity -- written to the sorted copies,
// which seeding and projection read -- and is integrated and collided again
// from there with the acceleration the force stage computed at its own
// position.
// ---------------------------------------------------------------------------
__global__ void k_ts_children(int n, float4* __restrict__ posS, float4* __restrict__ velS,
                              const float4* __restrict__ accS, const float4* __restrict__ rho4S,
                              const int* __restrict__ workIds, float mass, PhysDev ph, int collideFlag,
                              float4* __restrict__ pos, float4* __restrict__ vel, TwoScaleDev T) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int id = workIds[k];
    const unsigned int code = T.state[id] & 15u;
    const int was = state_class(code >> 2), now = state_class(code & 3u);
    if (T.childMode == 1 && was == 1 && now != 1) {
        float sx = 0.f, sy = 0.f, sz = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
        for (int c = 0; c < 8; c++) {
            const float4 a = T.subPos[8 * (size_t)id + c], b = T.subVel[8 * (size_t)id + c];
            sx = __fadd_rn(sx, a.x);
            sy = __fadd_rn(sy, a.y);
            sz = __fadd_rn(sz, a.z);
            ux = __fadd_rn(ux, b.x);
            uy = __fadd_rn(uy, b.y);
            uz = __fadd_rn(uz, b.z);
        }
        const float4 x0 = posS[k], v0 = velS[k];
        const float3 xm = make_float3(sx * 0.125f, sy * 0.125f, sz * 0.125f);
        const float3 vm = make_float3(ux * 0.125f, uy * 0.125f, uz * 0.125f);
        posS[k] = make_float4(xm.x, xm.y, xm.z, x0.w);
        velS[k] = make_float4(vm.x, vm.y, vm.z, v0.w);
        const float4 a = accS[k];
        float3 v = make_float3(vm.x + ph.dt * a.x, vm.y + ph.dt * a.y, vm.z + ph.dt * a.z);
        float3 x = make_float3(xm.x + ph.dt * v.x, xm.y + ph.dt * v.y, xm.z + ph.dt * v.z);
        if (collideFlag) collide(ph, x, v);
        pos[id] = make_float4(x.x, x.y, x.z, x0.w);
        vel[id] = make_float4(v.x, v.y, v.z, 0.f);
    }
    if ((code & 3u) == 0) return;
    // childMode 1: seed only on a class change (:1052-1055)
    if (T.childMode == 1 && was == now) return;
    const double rad = (double)(3.0f * mass) / (4.0 * 3.14159265358979323846 * (double)rho4S[k].x);
    const float radicand = (float)rad;
    const float radius = (float)pow((double)radicand, (double)(1.0f / 3.0f));
    const float4 x = posS[k], v = velS[k];
    const float d = (float)0.577350269;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float sx = (c & 4) ? -d : d, sy = (c & 2) ? -d : d, sz = (c & 1) ? -d : d;
        const size_t slot = 8 * (size_t)id + c;
        T.subPos[slot] = make_float4(__fmaf_rn(sx, radius, x.x), __fmaf_rn(sy, radius, x.y),
                                     __fmaf_rn(sz, radius, x.z), 0.f);
        T.subVel[slot] = make_float4(v.x, v.y, v.z, 0.f);
    }
}

// ---------------------------------------------------------------------------
// project_quantities (:570-622, 1328-1381): boundary children take the mean
// coarse density and pressure within compactSupportSub, searched on the
// coarse grid.  A child with nothing in reach gets 0 (the reference divides
// 0 by 0).  Coarse positions come from `coarsePos` in the working order, or
// through workIds from the particle-order state when `byId` is set.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TS_WARP_BLOCK) k_ts_project(const float4* __restrict__ coarsePos,
                                                              const int* __restrict__ workIds, int byId,
                                                              const float4* __restrict__ rho4S,
                                                              const int* __restrict__ cellOffset, GridDev g,
                                                              float hs, TwoScaleDev T) {
    const int first = 8 * T.counts[0];
    const int nSub = T.counts[3];
    const float hs2 = __fmul_rn(hs, hs);
    const int lane = threadIdx.x & 31, gl = lane & (TS_G - 1), grp = lane / TS_G;
    const int warps = gridDim.x * (TS_WARP_BLOCK / 32);
    constexpr int per = 32 / TS_G;
    for (int base = first + per * ((blockIdx.x * TS_WARP_BLOCK + threadIdx.x) >> 5); base < nSub;
         base += per * warps) {
        const int idx = base + grp;
        const bool valid = idx < nSub;
        const int slot = valid ? T.subIds[idx] : 0;
        const float4 x = valid ? T.subPos[slot] : make_float4(g.origin[0], g.origin[1], g.origin[2], 0.f);
        const GroupRows R = group_rows(group_stencil(x, hs, g, gl), g, cellOffset, gl, valid);
        float d = 0.f, p = 0.f, cnt = 0.f;
        for (int r = 0; r < 9; r++) {
            int s0, e;
            group_row(R, r, s0, e);
            for (int t = s0 + gl; t < e; t += TS_G * TS_GBATCH) {
                float4 xc[TS_GBATCH], rc[TS_GBATCH];
#pragma unroll
                for (int u = 0; u < TS_GBATCH; u++) {
                    const int c = t + TS_G * u;
                    if (c < e) {
                        xc[u] = byId ? __ldg(coarsePos + __ldg(workIds + c)) : __ldg(coarsePos + c);
                        rc[u] = __ldg(rho4S + c);
                    }
                }
#pragma unroll
                for (int u = 0; u < TS_GBATCH; u++)
                    if (t + TS_G * u < e && ref_r2(x, xc[u]) <= hs2) {
                        d += rc[u].x;
                        p += rc[u].y;
                        cnt += 1.f;
                    }
            }
        }
        d = group_total(d);
        p = group_total(p);
        cnt = group_total(cnt);
        if (valid && gl == 0) T.subRho[slot] = cnt > 0.f ? make_float2(d / cnt, p / cnt) : make_float2(0.f, 0.f);
    }
}

// ---------------------------------------------------------------------------
// The fine level's sort: compute_sub_particle_hash (:121-153) over the child
// list, then the same counting sort as the coarse level, stable in list order.
// ---------------------------------------------------------------------------
__global__ void k_ts_subhash(GridDev g, TwoScaleDev T, unsigned int* status) {
    const int nSub = T.counts[3];
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nSub; idx += gridDim.x * blockDim.x)
        hash_child(T.subPos[T.subIds[idx]], g, T, idx, status);
}

__global__ void k_ts_subscatter(TwoScaleDev T) {
    const int nSub = T.counts[3];
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nSub; idx += gridDim.x * blockDim.x) {
        const int2 ks = T.subKeySlot[idx];
        const int dst = T.subOffset[ks.x] + ks.y;
        T.subTmp[dst] = idx;
        T.subSortedHash[dst] = ks.x;
    }
}

__global__ void k_ts_subrank(TwoScaleDev T) {
    const int nSub = T.counts[3];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nSub; k += gridDim.x * blockDim.x) {
        const int c = T.subSortedHash[k];
        const int s = T.subOffset[c], e = T.subOffset[c + 1];
        const int my = T.subTmp[k];
        int r = 0;
        for (int t = s; t < e; t++) r += T.subTmp[t] < my;
        const int slot = T.subIds[my];
        T.subSortedIds[s + r] = slot;
        T.subPosS[s + r] = T.subPos[slot];
        T.subVelS[s + r] = T.subVel[slot];
    }
}

// ---------------------------------------------------------------------------
// compute_sub_particle_density_pressure (:259-313) for regular children.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TS_WARP_BLOCK) k_ts_subdensity(GridDev g, PhysDev ph, TwoScaleDev T) {
    const int nReg = 8 * T.counts[0];
    const int lane = threadIdx.x & 31, gl = lane & (TS_G - 1), grp = lane / TS_G;
    const int warps = gridDim.x * (TS_WARP_BLOCK / 32);
    constexpr int per = 32 / TS_G;
    for (int base = per * ((blockIdx.x * TS_WARP_BLOCK + threadIdx.x) >> 5); base < nReg; base += per * warps) {
        const int idx = base + grp;
        const bool valid = idx < nReg;
        const int slot = valid ? T.subIds[idx] : 0;
        const float4 x = valid ? T.subPos[slot] : make_float4(g.origin[0], g.origin[1], g.origin[2], 0.f);
        const GroupRows R = group_rows(group_stencil(x, ph.h, g, gl), g, T.subOffset, gl, valid);
        float sum = 0.f, comp = 0.f;
        for (int r = 0; r < 9; r++) {
            int s0, e;
            group_row(R, r, s0, e);
            float part = 0.f;
            for (int t = s0 + gl; t < e; t += TS_G * TS_GBATCH) {
                float4 xc[TS_GBATCH];
#pragma unroll
                for (int u = 0; u < TS_GBATCH; u++)
                    if (t + TS_G * u < e) xc[u] = __ldg(T.subPosS + t + TS_G * u);
#pragma unroll
                for (int u = 0; u < TS_GBATCH; u++)
                    if (t + TS_G * u < e) {
                        const float q = fmaxf(ph.h2 - dist2(x, xc[u]), 0.f);
                        part = fmaf(q * q, q, part);
                    }
            }
            // the row's sum, compensated over the rows in order
            const float rs = group_total(part);
            if (rs > 0.f) kahan_add(sum, comp, rs);
        }
        const float rho = __fsub_rn(sum, comp) * ph.poly6m;
        if (valid && gl == 0) T.subRho[slot] = make_float2(rho, ph.stiffness * (rho - ph.restDensity));
    }
}

// ---------------------------------------------------------------------------
// compute_sub_particle_acceleration (:477-568): pressure, viscosity and the
// colour field of the regular children; surface tension is always tested
// (no wall terms at this level).  Then integrate_sub_particles_euler
// (:667-696) + collision_handling_sub_particles (:836-930) for every child
// of the list, in the same launch: neighbours are read from the sorted
// copies only, so a child can be moved as soon as its own sums are done.
// Children of boundary particles use whatever acceleration their slot holds
// (the reference computes none for them).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void integrate_child(const PhysDev& ph, const TwoScaleDev& T, int slot, float4 a,
                                                float4 x0, float4 v0) {
    float3 v = make_float3(v0.x + ph.dt * a.x, v0.y + ph.dt * a.y, v0.z + ph.dt * a.z);
    float3 x = make_float3(x0.x + ph.dt * v.x, x0.y + ph.dt * v.y, x0.z + ph.dt * v.z);
    collide(ph, x, v);
    T.subPos[slot] = make_float4(x.x, x.y, x.z, 0.f);
    T.subVel[slot] = make_float4(v.x, v.y, v.z, 0.f);
}

// Hit queue of one group: a round adds at most TS_G * TS_GBATCH pairs to
// fewer than TS_G left over.
constexpr int TS_QUEUE = TS_G * TS_GBATCH + TS_G;

__global__ void __launch_bounds__(TS_WARP_BLOCK) k_ts_subforce(GridDev g, PhysDev ph, TwoScaleDev T) {
    __shared__ int s_queue[TS_WARP_BLOCK / TS_G][TS_QUEUE];
    const int nReg = 8 * T.counts[0];
    const int nSub = T.counts[3];
    for (int idx = nReg + blockIdx.x * TS_WARP_BLOCK + threadIdx.x; idx < nSub; idx += gridDim.x * TS_WARP_BLOCK) {
        const int slot = T.subIds[idx];
        integrate_child(ph, T, slot, T.subAcc[slot], T.subPos[slot], T.subVel[slot]);
    }
    const int lane = threadIdx.x & 31, gl = lane & (TS_G - 1), grp = lane / TS_G;
    const unsigned int below = (1u << gl) - 1u;
    int* queue = s_queue[threadIdx.x / TS_G];
    const int warps = gridDim.x * (TS_WARP_BLOCK / 32);
    constexpr int per = 32 / TS_G;
    for (int base = per * ((blockIdx.x * TS_WARP_BLOCK + threadIdx.x) >> 5); base < nReg; base += per * warps) {
        const int idx = base + grp;
        const bool valid = idx < nReg;
        const int slot = valid ? T.subIds[idx] : 0;
        const float4 xi = valid ? T.subPos[slot] : make_float4(g.origin[0], g.origin[1], g.origin[2], 0.f);
        const float4 vi = valid ? T.subVel[slot] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 ri = valid ? T.subRho[slot] : make_float2(1.f, 0.f);
        const float rhoi = ri.x;
        const float qi = ri.y / (rhoi * rhoi);
        const GroupRows R = group_rows(group_stencil(xi, ph.h, g, gl), g, T.subOffset, gl, valid);
        float fp[3] = {0.f, 0.f, 0.f}, fv[3] = {0.f, 0.f, 0.f}, cg[3] = {0.f, 0.f, 0.f}, cl = 0.f;
        auto pair = [&](int c) {
            const float4 xj = __ldg(T.subPosS + c), vj = __ldg(T.subVelS + c);
            const float2 rj = T.subRho[__ldg(T.subSortedIds + c)];
            const float r2 = dist2(xi, xj);
            const float invj = 1.0f / rj.x;
            const float dx = __fsub_rn(xi.x, xj.x), dy = __fsub_rn(xi.y, xj.y), dz = __fsub_rn(xi.z, xj.z);
            const float rinv = rsqrtf(r2);
            const float hr = ph.h - r2 * rinv;
            const float sp = (qi + rj.y * invj * invj) * hr * hr * rinv;
            const float sv = invj * hr;
            fp[0] = fmaf(sp, dx, fp[0]);
            fp[1] = fmaf(sp, dy, fp[1]);
            fp[2] = fmaf(sp, dz, fp[2]);
            fv[0] = fmaf(sv, vj.x - vi.x, fv[0]);
            fv[1] = fmaf(sv, vj.y - vi.y, fv[1]);
            fv[2] = fmaf(sv, vj.z - vi.z, fv[2]);
            const float d2 = ph.h2 - r2;
            const float sc = invj * d2 * d2;
            cg[0] = fmaf(sc, dx, cg[0]);
            cg[1] = fmaf(sc, dy, cg[1]);
            cg[2] = fmaf(sc, dz, cg[2]);
            cl = fmaf(invj * d2, 3.f * ph.h2 - 7.f * r2, cl);
        };
        // row by row, rounds of TS_GBATCH candidates per lane: test and list
        // the hits in the group's queue; the group's lanes take the listed
        // pairs TS_G at a time
        int listed = 0;
        for (int r = 0; r < 9; r++) {
            int s0, e;
            group_row(R, r, s0, e);
            for (int t = s0 + gl; __any_sync(0xffffffffu, t < e); t += TS_G * TS_GBATCH) {
                float4 xc[TS_GBATCH];
#pragma unroll
                for (int u = 0; u < TS_GBATCH; u++)
                    if (t + TS_G * u < e) xc[u] = __ldg(T.subPosS + t + TS_G * u);
#pragma unroll
                for (int u = 0; u < TS_GBATCH; u++) {
                    bool hit = false;
                    if (t + TS_G * u < e) {
                        const float r2 = dist2(xi, xc[u]);
                        hit = r2 <= ph.h2 && r2 > 0.f;
                    }
                    const unsigned int m = (__ballot_sync(0xffffffffu, hit) >> (TS_G * grp)) & 0xFFu;
                    if (hit) queue[listed + __popc(m & below)] = t + TS_G * u;
                    listed += __popc(m);
                }
                const int take = listed & ~(TS_G - 1);
                __syncwarp();
                for (int q = gl; q < take; q += TS_G) pair(queue[q]);
                // fewer than TS_G left: to the front of the queue
                const int left = listed - take;
                const int keep = gl < left ? queue[take + gl] : 0;
                __syncwarp();
                if (gl < left) queue[gl] = keep;
                listed = left;
                __syncwarp();
            }
        }
        if (gl < listed) pair(queue[gl]);
        __syncwarp();
        for (int a = 0; a < 3; a++) {
            fp[a] = group_total(fp[a]);
            fv[a] = group_total(fv[a]);
            cg[a] = group_total(cg[a]);
        }
        cl = group_total(cl);
        if (!valid || gl != 0) continue;
        const float pc = ph.pressCoef * rhoi;
        float force[3];
        for (int a = 0; a < 3; a++) force[a] = ph.viscCoef * fv[a] + pc * fp[a];
        const float cgx = ph.cgCoef * cg[0], cgy = ph.cgCoef * cg[1], cgz = ph.cgCoef * cg[2];
        const float norm = sqrtf(cgx * cgx + cgy * cgy + cgz * cgz);
        if (norm > ph.normThresh) {
            const float fc = ph.tension * (ph.clCoef * cl) / norm;
            force[0] -= fc * cgx;
            force[1] -= fc * cgy;
            force[2] -= fc * cgz;
        }
        float acc[3] = {force[0] / rhoi, force[1] / rhoi, force[2] / rhoi};
        acc[0] -= ph.gravityAxis == 0 ? ph.gravity : 0.f;
        acc[1] -= ph.gravityAxis == 1 ? ph.gravity : 0.f;
        acc[2] -= ph.gravityAxis == 2 ? ph.gravity : 0.f;
        const float4 a4 = make_float4(acc[0], acc[1], acc[2], 0.f);
        T.subAcc[slot] = a4;
        integrate_child(ph, T, slot, a4, xi, vi);
    }
}

// SD layout of the child slots (particle_simulation.h:28-41): mass and
// energy columns are never written by the reference (0).
__global__ void k_ts_pack_sd(TwoScaleDev T, int slots, float* __restrict__ dst) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= slots) return;
    float* o = dst + 10 * (size_t)k;
    const float2 r = T.subRho[k];
    const float4 a = T.subAcc[k], v = T.subVel[k];
    o[0] = 0.f;
    o[1] = r.x;
    o[2] = r.y;
    o[3] = a.x;
    o[4] = a.y;
    o[5] = a.z;
    o[6] = v.x;
    o[7] = v.y;
    o[8] = v.z;
    o[9] = 0.f;
}

}  // namespace

void launch_ts_pack_sd(const TwoScaleDev& T, int slots, float* dst, cudaStream_t s) {
    if (slots <= 0) return;
    k_ts_pack_sd<<<(slots + 255) / 256, 256, 0, s>>>(T, slots, dst);
}

void launch_ts_states(int n, const float4* posS, const int* workIds, const int* cellOffset, GridDev g, float h,
                      const TwoScaleDev& T, cudaStream_t s) {
    if (n <= 0) return;
    k_ts_state<<<(n + 255) / 256, 256, 0, s>>>(n, posS, workIds, T);
    k_ts_mark<<<warp_grid(n), TS_WARP_BLOCK, 0, s>>>(posS, workIds, cellOffset, g, h, T);
    const int nb = (n + TS_BLOCK - 1) / TS_BLOCK;
    k_ts_count<<<nb, TS_BLOCK, 0, s>>>(n, T);
    k_ts_lists<<<nb, TS_BLOCK, 0, s>>>(n, T);
}

void launch_ts_children(int n, float4* posS, float4* velS, const float4* accS, const float4* rho4S,
                        const int* workIds, float mass, PhysDev ph, int collide, float4* pos, float4* vel,
                        const TwoScaleDev& T, cudaStream_t s) {
    if (n <= 0) return;
    k_ts_children<<<(n + 127) / 128, 128, 0, s>>>(n, posS, velS, accS, rho4S, workIds, mass, ph, collide, pos, vel,
                                                  T);
}

void launch_ts_project(const float4* coarsePos, const int* workIds, int byId, const float4* rho4S,
                       const int* cellOffset, GridDev g, float hs, const TwoScaleDev& T, int capacity,
                       cudaStream_t s) {
    k_ts_project<<<group_grid(capacity), TS_WARP_BLOCK, 0, s>>>(coarsePos, workIds, byId, rho4S, cellOffset, g, hs,
                                                                T);
}

void launch_ts_sub_sort(GridDev sg, const TwoScaleDev& T, SortBuffers subSb, int capacity, unsigned int* status,
                        cudaStream_t s) {
    k_ts_subhash<<<stride_grid(capacity, 256), 256, 0, s>>>(sg, T, status);
    launch_cell_scan(sg.numCells, subSb, status, s);
    k_ts_subscatter<<<stride_grid(capacity, 256), 256, 0, s>>>(T);
    k_ts_subrank<<<stride_grid(capacity, 256), 256, 0, s>>>(T);
}

void launch_ts_sub_density(GridDev sg, PhysDev sph, const TwoScaleDev& T, int capacity, cudaStream_t s) {
    k_ts_subdensity<<<group_grid(capacity), TS_WARP_BLOCK, 0, s>>>(sg, sph, T);
}

void launch_ts_sub_force(GridDev sg, PhysDev sph, const TwoScaleDev& T, int capacity, cudaStream_t s) {
    k_ts_subforce<<<group_grid(capacity), TS_WARP_BLOCK, 0, s>>>(sg, sph, T);
}


}  // namespace sph
