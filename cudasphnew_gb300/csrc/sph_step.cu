// Density and force stages of the GB300 SPH step.
//
// Both run one thread per particle in the working order (cell, x, id) and
// walk the nine rows of the 27-cell stencil (sph_device.cuh), each cut to its
// candidate window.  Each row's terms are summed in plain FP32 (a row holds a
// handful of neighbours) and the row sums are added with Kahan compensation;
// a row that contributes exactly nothing is not added, so the window cut
// (which drops only zero terms) changes no result bit.
//
// The force stage comes in three forms that sum the same terms in the same
// order:
//   direct    -- distance test and pair interaction in one loop (the
//                reference's structure); a warp runs the interaction whenever
//                any lane's candidate is a neighbour;
//   mask      -- a row is tested in chunks of up to 32 candidates into a
//                register bit mask first, then only the set bits interact;
//   pretested -- the density stage, which tests every candidate anyway,
//                records each row's window start and a 32-bit neighbour mask;
//                the force stage runs the interactions of the set bits only
//                (rows longer than 32 candidates fall back to testing).
#include <climits>

#include "sph_device.cuh"
#include "sph_mlp_tile.cuh"

namespace sph {

// ---------------------------------------------------------------------------
// Density + pressure (compute_particle_density_pressure,
// particle_simulation.cu:196-256; compute_particle_density_cell :1385-1419).
// Branch-free poly6 accumulation: max(h^2 - r^2, 0)^3.  Writes
// (rho, p, p/rho^2, 1/rho) for the force stage.
// ---------------------------------------------------------------------------
struct RowMasks {
    int* start;          // [9][n] window start, bit 31 set when the row was not masked
    unsigned int* mask;  // [9][n] neighbour bits relative to start, or the window end
};

// With REL the positions are cell-relative: every neighbour is moved into
// particle i's cell frame before its distance is taken.
// Occupancy: 40 registers (six 256-thread blocks per SM) cost no spills
// outside the batched form's setup, and the stage runs ~1 % faster than at
// 48; the cell-relative forms keep 48.
template <bool KAHAN, bool EMIT, bool BATCH, bool REL>
__global__ void __launch_bounds__(256, REL ? 5 : 6)
k_density(int n, const float4* __restrict__ posS, RowTables T, GridDev g_, PhysDev ph_, MapDev map_, int window,
          float4* __restrict__ rho4S, RowMasks M) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (T.skip && *T.skip)) return;
    const float4 xi = posS[i];
    // batched handles: the particle's own scene supplies grid, constants and maps
    const SceneDev* S = BATCH ? T.scenes + __float_as_int(xi.w) : nullptr;
    const GridDev& g = BATCH ? S->g : g_;
    const PhysDev& ph = BATCH ? S->ph : ph_;
    const MapDev& map = BATCH ? S->map : map_;
    const int3 ci = REL ? rel_cell(xi) : make_int3(0, 0, 0);
    const Stencil st = REL ? stencil_rel(xi, ci, ph.h, g) : stencil(xi, ph.h, g);
    const float h2 = ph.h2;
    float sum = 0.f, comp = 0.f;
#pragma unroll
    for (int r = 0; r < 9; r++) {
        int s, e;
        float dyo = 0.f, dzo = 0.f;
        if (REL) row_range_rel(xi, ci, st, ph.h, g, T, window != 0, r, s, e, dyo, dzo);
        else row_range(xi, st, ph.h, g, T, window != 0, r, s, e);
        float rs = 0.f;
        // neighbour bits, first candidate in the highest bit used (one
        // multiply-add per candidate), turned around after the row; two
        // candidates per loop turn (176 -> 172 us per million particles;
        // four gain nothing more)
        unsigned int m = 0u;
#pragma unroll 2
        for (int t = s; t < e; t++) {
            float4 xj = __ldg(posS + t);
            if (REL) xj = rel_in_frame(xj, ci.x, dyo, dzo, g.spacing);
            const float r2 = dist2(xi, xj);
            const float w = fmaxf(h2 - r2, 0.f);
            rs = fmaf(w * w, w, rs);
            if (EMIT) m = m * 2u + (neighbour_r2(r2, h2) ? 1u : 0u);
        }
        if (KAHAN) {
            if (rs > 0.f) kahan_add(sum, comp, rs);
        } else {
            sum += rs;
        }
        if (EMIT) {
            const int c = e - s;
            const bool fits = c <= 32;
            const unsigned int bits = (fits && c > 0) ? __brev(m) >> (32 - c) : 0u;  // bit k: candidate s + k
            M.start[(size_t)r * n + i] = fits ? s : (s | (int)0x80000000);
            M.mask[(size_t)r * n + i] = fits ? bits : (unsigned int)e;
        }
    }
    float rho = (KAHAN ? __fsub_rn(sum, comp) : sum) * ph.poly6m;
    if (map.present) {
        float uvw[3];
        map_uvw(map, REL ? rel_abs(xi, ci, g) : xi, uvw);
        rho += tri_vec(map, uvw[0], uvw[1], uvw[2]).y;  // wall density, :242-248
    }
    const float p = ph.stiffness * (rho - ph.restDensity);
    const float inv = 1.0f / rho;
    rho4S[i] = make_float4(rho, p, p * inv * inv, inv);
}

// ---------------------------------------------------------------------------
// Density over reused neighbour lists (sph_options.neighbourSkin).
//
// Build form (steps that build the lists): the reference's 3 x 3 stencil
// rows first, in its order, into slots 0-8, then the further rows the skin
// sphere of radius R reaches; each row's window at R is walked in the working
// order and the density terms are summed as in k_density (candidates beyond
// h add exactly nothing, so the reference's rows give the same row sums).
// Each row is recorded with two 64-bit masks over its candidates, starting at
// its first candidate within R: the candidates within R (the lists) and the
// neighbours within h (this step's force stage).  A row whose candidates
// within R span more than 64 places is kept unmasked.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool within_r2(float r2, float R2) {  // r2 >= 0 or NaN
    return __float_as_uint(r2) <= __float_as_uint(R2);
}

// BATCH: the slot's scene supplies grid, constants, maps, R and the scene's
// own decision.
template <bool KAHAN, bool BATCH>
__device__ __forceinline__ void density_build_one(int i, int n, float4* posS, float4* velS, const RowTables& T,
                                                  const GridDev& g_, const PhysDev& ph_, const MapDev& map_,
                                                  float4* __restrict__ rho4S, const NeighbourLists& L) {
    const int scene = BATCH ? L.slotScene[i] : 0;
    if (!L.flags[VL_BUILD_NOW * L.numScenes + scene]) return;
    const float4 xi = posS[i];
    const SceneDev* S = BATCH ? T.scenes + scene : nullptr;
    const GridDev& g = BATCH ? S->g : g_;
    const PhysDev& ph = BATCH ? S->ph : ph_;
    const MapDev& map = BATCH ? S->map : map_;
    const Stencil st = stencil(xi, ph.h, g);
    const float R = BATCH ? (1.0f + L.skinFrac) * ph.h : L.radius;
    const float h2 = ph.h2, R2 = BATCH ? R * R : L.radius2, eps = 1e-3f * ph.h;
    float sum = 0.f, comp = 0.f;
    int extra = VL_INNER;  // next slot of a further row
    // `slot` >= 0: a fixed slot, written even when the row is empty
    auto visit = [&](int y, int z, int slot) {
        int s0 = 0, e0 = 0;
        const bool any = y >= 0 && row_window(xi, y, z, R, eps, g, T, s0, e0);
        float rs = 0.f;
        unsigned long long ms = 0ull, me = 0ull;  // bit t - first, for the first 64
        int first = -1, last = -1;
        if (any) {
            for (int t = s0; t < e0; t++) {
                const float4 xj = __ldg(posS + t);
                const float r2 = dist2(xi, xj);
                const float w = fmaxf(h2 - r2, 0.f);
                rs = fmaf(w * w, w, rs);
                if (within_r2(r2, R2)) {
                    if (first < 0) first = t;
                    last = t;
                    const int k = t - first;
                    if (k < 64) {
                        ms |= 1ull << k;
                        if (neighbour_r2(r2, h2)) me |= 1ull << k;
                    }
                }
            }
        }
        if (KAHAN) {
            if (rs > 0.f) kahan_add(sum, comp, rs);
        } else {
            sum += rs;
        }
        if (slot < 0) {
            if (first < 0 || extra >= VL_SLOTS) return;  // nothing within R to record
            slot = extra++;
        }
        const size_t at = (size_t)slot * n + i;
        if (first < 0) {
            L.start[at] = 0;
            L.skin[at] = make_uint2(0u, 0u);
            L.exact[at] = make_uint2(0u, 0u);
        } else if (last - first < 64) {
            L.start[at] = first;
            L.skin[at] = make_uint2((unsigned int)ms, (unsigned int)(ms >> 32));
            L.exact[at] = make_uint2((unsigned int)me, (unsigned int)(me >> 32));
        } else {
            L.start[at] = first | (int)0x80000000;
            L.skin[at] = make_uint2((unsigned int)(last + 1), 0u);
            L.exact[at] = make_uint2((unsigned int)(last + 1), 0u);
        }
    };
    // the reference's rows (k_density's order) into their slots, then the rest within R
    const int y1 = min(st.y1, st.y0 + 2), z1 = min(st.z1, st.z0 + 2);
#pragma unroll 1
    for (int r = 0; r < VL_INNER; r++) {
        const int z = st.z0 + r / 3, y = st.y0 + r % 3;
        visit(z <= z1 && y <= y1 ? y : -1, z, r);
    }
    int ya, yb, za, zb;
    cell_span(xi.y, R + eps, g, 1, ya, yb);
    cell_span(xi.z, R + eps, g, 2, za, zb);
#pragma unroll 1
    for (int z = za; z <= zb; z++)
#pragma unroll 1
        for (int y = ya; y <= yb; y++)
            if (z < st.z0 || z > z1 || y < st.y0 || y > y1) visit(y, z, -1);
    L.rows[i] = (unsigned char)extra;
    L.posB[i] = xi;
    float rho = (KAHAN ? __fsub_rn(sum, comp) : sum) * ph.poly6m;
    if (map.present) {
        float uvw[3];
        map_uvw(map, xi, uvw);
        rho += tri_vec(map, uvw[0], uvw[1], uvw[2]).y;  // wall density, :242-248
    }
    const float p = ph.stiffness * (rho - ph.restDensity);
    const float inv = 1.0f / rho;
    rho4S[i] = make_float4(rho, p, p * inv * inv, inv);
    // what the force stage needs of a neighbour besides its position and
    // velocity rides in their unused fourth lanes: two loads per pair, not three
    posS[i].w = p * inv * inv;
    velS[i].w = inv;
}

// (A grid of one wave striding over the particles would make the early
// return cheaper, but the build itself ran 15 % slower that way.)
template <bool KAHAN, bool BATCH>
__global__ void __launch_bounds__(256, 4)
k_density_build(int n, float4* posS, float4* velS, RowTables T, GridDev g, PhysDev ph, MapDev map,
                float4* __restrict__ rho4S, NeighbourLists L) {
    if (!BATCH && !L.flags[VL_BUILD_NOW]) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        density_build_one<KAHAN, BATCH>(i, n, posS, velS, T, g, ph, map, rho4S, L);
}

// List form: each recorded row's candidates within R, in the recorded order;
// the row's neighbours within h of this step are recorded for the force
// stage over the same window (empty and unmasked rows keep what the build
// wrote).  The next row's entries are loaded before the current row is walked.
template <bool KAHAN, bool BATCH>
__global__ void __launch_bounds__(256, 8)
k_density_lists(int n, float4* posS, float4* velS, PhysDev ph_, MapDev map_, float4* __restrict__ rho4S,
                NeighbourLists L, const SceneDev* __restrict__ scenes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int scene = BATCH ? L.slotScene[i] : 0;
    if (L.flags[VL_BUILD_NOW * L.numScenes + scene]) return;
    const float4 xi = posS[i];
    const PhysDev& ph = BATCH ? scenes[scene].ph : ph_;
    const MapDev& map = BATCH ? scenes[scene].map : map_;
    const float h2 = ph.h2;
    const int rows = L.rows[i];
    float sum = 0.f, comp = 0.f;
    int svN = __ldg(L.start + i);
    uint2 mN = __ldg(L.skin + i);
#pragma unroll 1
    for (int r = 0; r < rows; r++) {
        const int sv = svN;
        const uint2 m = mN;
        if (r + 1 < rows) {
            svN = __ldg(L.start + (size_t)(r + 1) * n + i);
            mN = __ldg(L.skin + (size_t)(r + 1) * n + i);
        }
        float rs = 0.f;
        if (sv < 0) {
            for (int t = sv & 0x7fffffff; t < (int)m.x; t++) {
                const float w = fmaxf(h2 - dist2(xi, __ldg(posS + t)), 0.f);
                rs = fmaf(w * w, w, rs);
            }
        } else if (m.x | m.y) {
            unsigned int e0 = 0u, e1 = 0u;
            unsigned int b = m.x;
            while (b) {
                const int k = __ffs(b) - 1;
                b &= b - 1u;
                const float r2 = dist2(xi, __ldg(posS + sv + k));
                const float w = fmaxf(h2 - r2, 0.f);
                rs = fmaf(w * w, w, rs);
                if (neighbour_r2(r2, h2)) e0 |= 1u << k;
            }
            b = m.y;
            while (b) {
                const int k = __ffs(b) - 1;
                b &= b - 1u;
                const float r2 = dist2(xi, __ldg(posS + sv + 32 + k));
                const float w = fmaxf(h2 - r2, 0.f);
                rs = fmaf(w * w, w, rs);
                if (neighbour_r2(r2, h2)) e1 |= 1u << k;
            }
            L.exact[(size_t)r * n + i] = make_uint2(e0, e1);
        }
        if (KAHAN) {
            if (rs > 0.f) kahan_add(sum, comp, rs);
        } else {
            sum += rs;
        }
    }
    float rho = (KAHAN ? __fsub_rn(sum, comp) : sum) * ph.poly6m;
    if (map.present) {
        float uvw[3];
        map_uvw(map, xi, uvw);
        rho += tri_vec(map, uvw[0], uvw[1], uvw[2]).y;  // wall density, :242-248
    }
    const float p = ph.stiffness * (rho - ph.restDensity);
    const float inv = 1.0f / rho;
    rho4S[i] = make_float4(rho, p, p * inv * inv, inv);
    // what the force stage needs of a neighbour besides its position and
    // velocity rides in their unused fourth lanes: two loads per pair, not three
    posS[i].w = p * inv * inv;
    velS[i].w = inv;
}

// ---------------------------------------------------------------------------
// Pair interaction (compute_viscosity_pressure_forces_and_ifsurf_cell,
// :1459-1556), per-row partial sums, compensated totals.
// ---------------------------------------------------------------------------
// The quantities of one pair (i, j) both the force sums and the feature
// sums use: offset, r^2, 1/r, h - r and the velocity difference v_j - v_i.
struct Pair {
    float dx, dy, dz, r2, rinv, hr, ux, uy, uz;
    __device__ __forceinline__ Pair(const PhysDev& ph, float4 xi, float4 vi, float4 xj, float4 vj) {
        dx = __fsub_rn(xi.x, xj.x);
        dy = __fsub_rn(xi.y, xj.y);
        dz = __fsub_rn(xi.z, xj.z);
        r2 = dist2(xi, xj);
        rinv = rsqrtf(r2);
        hr = ph.h - r2 * rinv;
        ux = vj.x - vi.x;
        uy = vj.y - vi.y;
        uz = vj.z - vi.z;
    }
};

template <bool TENSION>
struct RowSums {
    float fp[3], fv[3], cg[3], cl;
    int hits;
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int a = 0; a < 3; a++) fp[a] = fv[a] = cg[a] = 0.f;
        cl = 0.f;
        hits = 0;
    }
    // COUNT: count the pair here (a caller walking a neighbour mask adds the
    // mask's population once instead)
    template <bool COUNT = true>
    __device__ __forceinline__ void add(const PhysDev& ph, const Pair& p, float qi, float4 rj) {
        const float sp = (qi + rj.z) * p.hr * p.hr * p.rinv;  // (p_i/rho_i^2 + p_j/rho_j^2)(h-r)^2/r
        const float sv = rj.w * p.hr;                         // (h-r)/rho_j
        fp[0] = fmaf(sp, p.dx, fp[0]);
        fp[1] = fmaf(sp, p.dy, fp[1]);
        fp[2] = fmaf(sp, p.dz, fp[2]);
        fv[0] = fmaf(sv, p.ux, fv[0]);
        fv[1] = fmaf(sv, p.uy, fv[1]);
        fv[2] = fmaf(sv, p.uz, fv[2]);
        if (TENSION) {
            const float d2 = ph.h2 - p.r2;
            const float sc = rj.w * d2 * d2;
            cg[0] = fmaf(sc, p.dx, cg[0]);
            cg[1] = fmaf(sc, p.dy, cg[1]);
            cg[2] = fmaf(sc, p.dz, cg[2]);
            cl = fmaf(rj.w * d2, 3.f * ph.h2 - 7.f * p.r2, cl);
        }
        if (COUNT) hits++;
    }
    __device__ __forceinline__ void add(const PhysDev& ph, float4 xi, float4 vi, float qi, float4 xj, float4 vj,
                                        float4 rj) {
        add(ph, Pair(ph, xi, vi, xj, vj), qi, rj);
    }
};

// Neighbour sums of the learned corrector's input features (FEAT forms
// only; the scale factors poly6*m and m*gradSpiky are applied once at the
// end).  The neighbour count is the force sums' hit count.
struct FeatSums {
    float shep = 0.f, m1[3] = {0.f, 0.f, 0.f}, div = 0.f, curl[3] = {0.f, 0.f, 0.f}, cg[3] = {0.f, 0.f, 0.f};
    int cnt = 0;
    __device__ __forceinline__ void add(const PhysDev& ph, const Pair& p, float4 rj) {
        const float q = ph.h2 - p.r2;
        const float w = q * q * q * rj.w;              // W_ij / (poly6 m) * m/rho_j
        const float gs = p.hr * p.hr * p.rinv * rj.w;  // |gradW_ij| / (m gradSpiky) * m/rho_j / r
        shep += w;
        m1[0] = fmaf(w, p.ux, m1[0]);
        m1[1] = fmaf(w, p.uy, m1[1]);
        m1[2] = fmaf(w, p.uz, m1[2]);
        cg[0] = fmaf(gs, p.dx, cg[0]);
        cg[1] = fmaf(gs, p.dy, cg[1]);
        cg[2] = fmaf(gs, p.dz, cg[2]);
        div = fmaf(gs, p.ux * p.dx + p.uy * p.dy + p.uz * p.dz, div);   // u . d
        curl[0] = fmaf(gs, p.uy * p.dz - p.uz * p.dy, curl[0]);        // u x d
        curl[1] = fmaf(gs, p.uz * p.dx - p.ux * p.dz, curl[1]);
        curl[2] = fmaf(gs, p.ux * p.dy - p.uy * p.dx, curl[2]);
    }
};

// Where the force stage writes the features: feat[(byId ? workIds[i] : i) * 24].
struct FeatOut {
    float* feat;
    int byId;
    int boxWalls;
    float dtL;
};

template <bool KAHAN, bool TENSION>
struct ForceTotals {
    float fp[3] = {0.f, 0.f, 0.f}, cp[3] = {0.f, 0.f, 0.f};
    float fv[3] = {0.f, 0.f, 0.f}, cv[3] = {0.f, 0.f, 0.f};
    float cg[3] = {0.f, 0.f, 0.f}, cl = 0.f;
    __device__ __forceinline__ void add(const RowSums<TENSION>& r) {
        if (r.hits == 0) return;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (KAHAN) {
                kahan_add(fp[a], cp[a], r.fp[a]);
                kahan_add(fv[a], cv[a], r.fv[a]);
            } else {
                fp[a] += r.fp[a];
                fv[a] += r.fv[a];
            }
            if (TENSION) cg[a] += r.cg[a];
        }
        if (TENSION) cl += r.cl;
    }
};

// The 24 input features of the learned step corrector:
//   0 rho/rho0 - 1;  1 Shepard sum sum_j (m/rho_j) W_ij;  2-4 v;  5-7 a/g;
//   8-10 sum_j (m/rho_j) W_ij (v_j - v_i);  11 dtL sum_j (m/rho_j)(v_j - v_i).gradW_ij;
//   12-14 dtL sum_j (m/rho_j)(v_j - v_i) x gradW_ij;  15-17 h sum_j (m/rho_j) gradW_ij;
//   18 neighbours/32;  19 wall distance/h (box walls and boundary map, capped at 4);
//   20-22 unit wall normal into the fluid;  23 |v| dtL/h.
// W is poly6, gradW the spiky gradient, sums over neighbours within h of
// the pre-step state.  No reference counterpart.
__device__ __forceinline__ void feature_values(const FeatSums& fs, int boxWalls, float dtL, float4 xi, float4 vi,
                                               float4 ri, const float* acc, float mapDist, const float* mapN,
                                               const PhysDev& ph, float* f) {
    const float h = ph.h;
    float dw = 4.f * h, nx = 0.f, ny = 0.f, nz = 0.f;
    if (boxWalls) {
        const float c[3] = {xi.x - ph.boxCen[0], xi.y - ph.boxCen[1], xi.z - ph.boxCen[2]};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float da = ph.boxDim[a] - fabsf(c[a]);
            if (da < dw) {
                dw = da;
                const float sg = c[a] > 0.f ? -1.f : 1.f;
                nx = a == 0 ? sg : 0.f;
                ny = a == 1 ? sg : 0.f;
                nz = a == 2 ? sg : 0.f;
            }
        }
    }
    if (mapDist < dw) {
        dw = mapDist;
        nx = mapN[0];
        ny = mapN[1];
        nz = mapN[2];
    }
    dw = fminf(fmaxf(dw, 0.f), 4.f * h);
    const float gInv = ph.gravity != 0.f ? 1.f / ph.gravity : 1.f;
    const float gw = -ph.pressCoef;  // m gradSpiky
    const float kd = gw * dtL;
    const float vn = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z);
    f[0] = ri.x / ph.restDensity - 1.f;
    f[1] = ph.poly6m * fs.shep;
    f[2] = vi.x;
    f[3] = vi.y;
    f[4] = vi.z;
    f[5] = acc[0] * gInv;
    f[6] = acc[1] * gInv;
    f[7] = acc[2] * gInv;
    f[8] = ph.poly6m * fs.m1[0];
    f[9] = ph.poly6m * fs.m1[1];
    f[10] = ph.poly6m * fs.m1[2];
    f[11] = kd * fs.div;
    f[12] = kd * fs.curl[0];
    f[13] = kd * fs.curl[1];
    f[14] = kd * fs.curl[2];
    f[15] = gw * h * fs.cg[0];
    f[16] = gw * h * fs.cg[1];
    f[17] = gw * h * fs.cg[2];
    f[18] = (float)fs.cnt * (1.f / 32.f);
    f[19] = dw / h;
    f[20] = nx;
    f[21] = ny;
    f[22] = nz;
    f[23] = vn * dtL / h;
}

__device__ __forceinline__ void store_features(float* feat, size_t row, const float* f) {
    float4* dst = reinterpret_cast<float4*>(feat + row * 24);
#pragma unroll
    for (int c = 0; c < 6; c++) dst[c] = make_float4(f[4 * c], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3]);
}

// Wall terms, surface tension, a = F/rho - g, symplectic Euler, box
// collision, and the write-back (compute_particle_acceleration_ifsurf
// :407-473, integrate_euler :632-665, collision_handling :742-834).  The wall
// terms follow the reference's operation order exactly.
// Returns the new state (x, v) and the acceleration; the FEAT forms also
// return the boundary map's wall distance and unit normal (mapDist stays as
// given where the map is absent, mapN where the particle is beyond the
// map's rest distance).  xm is the absolute position the boundary map is
// read at (xi itself unless positions are cell-relative).
template <bool KAHAN, bool TENSION, bool FEAT>
__device__ __forceinline__ void force_finish(const ForceTotals<KAHAN, TENSION>& A, float4 xi, float4 vi, float4 ri,
                                             const PhysDev& ph, const MapDev& map, int collideFlag, float3& x,
                                             float3& v, float* acc, float& mapDist, float* mapN, float4 xm) {
    const float rho = ri.x;
    const float pc = ph.pressCoef * rho;
    float force[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float P = KAHAN ? __fsub_rn(A.fp[a], A.cp[a]) : A.fp[a];
        const float V = KAHAN ? __fsub_rn(A.fv[a], A.cv[a]) : A.fv[a];
        force[a] = ph.viscCoef * V + pc * P;
    }
    bool tension = TENSION;
    if (map.present) {
        float uvw[3];
        map_uvw(map, xm, uvw);
        const float4 s = tri_vec(map, uvw[0], uvw[1], uvw[2]);
        const float distWall = -s.x;
        if (FEAT) mapDist = distWall;
        if (distWall < map.restDistance) {
            tension = false;
            const float coeff = rho / (ph.dtCollide * ph.dtCollide) * (map.restDistance - distWall);
            float gN[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                float up[3] = {uvw[0], uvw[1], uvw[2]}, dn[3] = {uvw[0], uvw[1], uvw[2]};
                up[a] = __fadd_rn(uvw[a], map.du[a]);
                dn[a] = __fsub_rn(uvw[a], map.du[a]);
                gN[a] = __fdiv_rn(__fsub_rn(tri_scalar(map, map.dist, up[0], up[1], up[2]),
                                            tri_scalar(map, map.dist, dn[0], dn[1], dn[2])),
                                  __fmul_rn(2.f, map.du[a]));
            }
            force[0] -= coeff * gN[0];
            force[1] -= coeff * gN[1];
            force[2] -= coeff * gN[2];
            if (FEAT) {
                const float gn = sqrtf(gN[0] * gN[0] + gN[1] * gN[1] + gN[2] * gN[2]);
                if (gn > 0.f) {
                    mapN[0] = -gN[0] / gn;
                    mapN[1] = -gN[1] / gn;
                    mapN[2] = -gN[2] / gn;
                }
            }
            force[0] -= vi.x * s.z;
            force[1] -= vi.y * s.z;
            force[2] -= vi.z * s.z;
        }
    }
    if (TENSION && tension) {
        const float cgx = ph.cgCoef * A.cg[0], cgy = ph.cgCoef * A.cg[1], cgz = ph.cgCoef * A.cg[2];
        const float norm = sqrtf(cgx * cgx + cgy * cgy + cgz * cgz);
        if (norm > ph.normThresh) {
            const float fc = ph.tension * (ph.clCoef * A.cl) / norm;
            force[0] -= fc * cgx;
            force[1] -= fc * cgy;
            force[2] -= fc * cgz;
        }
    }
    acc[0] = force[0] / rho;
    acc[1] = force[1] / rho;
    acc[2] = force[2] / rho;
    acc[0] -= ph.gravityAxis == 0 ? ph.gravity : 0.f;
    acc[1] -= ph.gravityAxis == 1 ? ph.gravity : 0.f;
    acc[2] -= ph.gravityAxis == 2 ? ph.gravity : 0.f;
    v = make_float3(vi.x + ph.dt * acc[0], vi.y + ph.dt * acc[1], vi.z + ph.dt * acc[2]);
    x = make_float3(xi.x + ph.dt * v.x, xi.y + ph.dt * v.y, xi.z + ph.dt * v.z);
    if (collideFlag) collide(ph, x, v);
}

template <bool KAHAN, bool TENSION, bool FEAT>
__device__ __forceinline__ void force_epilogue(const ForceTotals<KAHAN, TENSION>& A, int i, float4 xi,
                                               float4 vi, float4 ri, const PhysDev& ph, const MapDev& map,
                                               int collideFlag, const int* __restrict__ workIds,
                                               float4* __restrict__ pos, float4* __restrict__ vel,
                                               float4* __restrict__ accS, const FeatSums& fs,
                                               const FeatOut& fo) {
    float mapDist = 1e30f, mapN[3] = {0.f, 0.f, 0.f};  // learned features only
    float3 x, v;
    float acc[3];
    force_finish<KAHAN, TENSION, FEAT>(A, xi, vi, ri, ph, map, collideFlag, x, v, acc, mapDist, mapN, xi);
    const int id = workIds[i];
    pos[id] = make_float4(x.x, x.y, x.z, xi.w);  // .w: the scene index of batched handles
    vel[id] = make_float4(v.x, v.y, v.z, 0.f);
    accS[i] = make_float4(acc[0], acc[1], acc[2], 0.f);
    if (FEAT) {
        float f[24];
        feature_values(fs, fo.boxWalls, fo.dtL, xi, vi, ri, acc, mapDist, mapN, ph, f);
        store_features(fo.feat, (size_t)(fo.byId ? id : i), f);
    }
}

// The cell-relative form's epilogue: the step is integrated in the
// particle's cell frame, then the position moves to the cell it now lies in
// (whole-cell steps, clamped to the grid).  The wall box collision works in
// that cell's frame too, and a particle it moves is re-binned again.
__device__ __forceinline__ void rel_rebin(float3& x, int3& c, const GridDev& g) {
    const float inv = 1.0f / g.spacing;
    float* xs[3] = {&x.x, &x.y, &x.z};
    int* cs[3] = {&c.x, &c.y, &c.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float k = floorf(*xs[a] * inv);
        if (k != 0.f) {
            const int cn = min(max(*cs[a] + (int)k, 0), g.dim[a] - 1);
            *xs[a] = fmaf(-(float)(cn - *cs[a]), g.spacing, *xs[a]);
            *cs[a] = cn;
        }
    }
}

template <bool KAHAN, bool TENSION>
__device__ __forceinline__ void force_epilogue_rel(const ForceTotals<KAHAN, TENSION>& A, int i, float4 xi, int3 ci,
                                                   float4 vi, float4 ri, const PhysDev& ph, const GridDev& g,
                                                   const MapDev& map, int collideFlag, const int* __restrict__ workIds,
                                                   float4* __restrict__ pos, float4* __restrict__ vel,
                                                   float4* __restrict__ accS) {
    float mapDist = 1e30f, mapN[3] = {0.f, 0.f, 0.f};
    float3 x, v;
    float acc[3];
    force_finish<KAHAN, TENSION, false>(A, xi, vi, ri, ph, map, 0, x, v, acc, mapDist, mapN, rel_abs(xi, ci, g));
    int3 c = ci;
    rel_rebin(x, c, g);
    if (collideFlag) {
        // the wall box in this cell's frame: the collision keeps the offset's resolution
        const int cc[3] = {c.x, c.y, c.z};
        float cen[3];
#pragma unroll
        for (int a = 0; a < 3; a++)
            cen[a] = (float)((double)ph.boxCen[a] - ((double)g.origin[a] + (double)cc[a] * (double)g.spacing));
        const float3 before = x;
        collide_box(cen, ph, x, v);
        if (x.x != before.x || x.y != before.y || x.z != before.z) rel_rebin(x, c, g);
    }
    const int id = workIds[i];
    pos[id] = make_float4(x.x, x.y, x.z, rel_pack(c.x, c.y, c.z));
    vel[id] = make_float4(v.x, v.y, v.z, 0.f);
    accS[i] = make_float4(acc[0], acc[1], acc[2], 0.f);
}

struct ForceArgs {
    int n;
    const float4* posS;
    const float4* velS;
    const float4* rho4S;
    const int* workIds;
    RowTables T;
    GridDev g;
    PhysDev ph;
    MapDev map;
    int collide;
    int window;
    RowMasks M;
    float4* pos;
    float4* vel;
    float4* accS;
    FeatOut fo;
};

// Occupancy: the force stage is latency bound, so it runs as many warps as
// fit without heavy spilling.  The pretested form without surface tension
// fits 48 registers with a few spilled bytes outside the pair loop: five
// 256-thread blocks per SM (145 -> 140 us per million particles against
// four).  The other plain forms and the batched forms fit 64 registers, four
// blocks (210 -> 150 us against two; the 64-scene batch 1.55 -> 1.44 ms per
// step against three); the feature form takes up to 80, three blocks.
// REL: cell-relative positions (plain forms only): neighbours are moved into
// particle i's cell frame, the step is integrated there and re-binned.
template <bool KAHAN, bool TENSION, int FORM, bool FEAT, bool BATCH, bool REL = false>
__global__ void __launch_bounds__(256, FEAT ? 3 : (BATCH || TENSION || REL || FORM != FORCE_PRETESTED ? 4 : 5)) k_force(ForceArgs F) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n) return;
    const float4 xi = F.posS[i];
    const float4 vi = F.velS[i];
    const float4 ri = F.rho4S[i];
    const SceneDev* S = BATCH ? F.T.scenes + __float_as_int(xi.w) : nullptr;
    const GridDev& g = BATCH ? S->g : F.g;
    const PhysDev& ph = BATCH ? S->ph : F.ph;
    const MapDev& map = BATCH ? S->map : F.map;
    const float h2 = ph.h2;
    const int3 ci = REL ? rel_cell(xi) : make_int3(0, 0, 0);
    Stencil st;
    if (REL) st = stencil_rel(xi, ci, ph.h, g);
    else if (FORM != FORCE_PRETESTED) st = stencil(xi, ph.h, g);
    float dyo = 0.f, dzo = 0.f;  // REL: the current row's y and z cell offsets (times spacing)
    auto neighbour = [&](int t) {
        float4 xj = __ldg(F.posS + t);
        if (REL) xj = rel_in_frame(xj, ci.x, dyo, dzo, g.spacing);
        return xj;
    };
    ForceTotals<KAHAN, TENSION> A;
    FeatSums fs;
    auto direct = [&](RowSums<TENSION>& R, int s, int e) {
        for (int t = s; t < e; t++) {
            const float4 xj = neighbour(t);
            const float r2 = dist2(xi, xj);
            if (neighbour_r2(r2, h2)) {
                const float4 vj = __ldg(F.velS + t), rj = __ldg(F.rho4S + t);
                const Pair p(ph, xi, vi, xj, vj);
                R.add(ph, p, ri.z, rj);
                if (FEAT) fs.add(ph, p, rj);
            }
        }
    };
    auto bits = [&](RowSums<TENSION>& R, int base, unsigned int m) {
        R.hits += __popc(m);
        while (m) {
            const int t = base + __ffs(m) - 1;
            m &= m - 1u;
            const float4 xj = neighbour(t), vj = __ldg(F.velS + t), rj = __ldg(F.rho4S + t);
            const Pair p(ph, xi, vi, xj, vj);
            R.template add<false>(ph, p, ri.z, rj);
            if (FEAT) fs.add(ph, p, rj);
        }
    };
#pragma unroll
    for (int r = 0; r < 9; r++) {
        RowSums<TENSION> R;
        R.clear();
        if (FORM == FORCE_PRETESTED) {
            if (REL) {
                dyo = (float)(st.y0 + r % 3 - ci.y) * g.spacing;
                dzo = (float)(st.z0 + r / 3 - ci.z) * g.spacing;
            }
            const int sv = __ldg(F.M.start + (size_t)r * F.n + i);
            const unsigned int m = __ldg(F.M.mask + (size_t)r * F.n + i);
            if (sv < 0) direct(R, sv & 0x7fffffff, (int)m);
            else bits(R, sv, m);
        } else {
            int s, e;
            if (REL) row_range_rel(xi, ci, st, ph.h, g, F.T, F.window != 0, r, s, e, dyo, dzo);
            else row_range(xi, st, ph.h, g, F.T, F.window != 0, r, s, e);
            if (FORM == FORCE_DIRECT) {
                direct(R, s, e);
            } else {
                for (int base = s; base < e; base += 32) {
                    const int cnt = min(32, e - base);
                    unsigned int m = 0u;
                    for (int k = 0; k < cnt; k++) {
                        const float r2 = dist2(xi, neighbour(base + k));
                        m |= neighbour_r2(r2, h2) ? (1u << k) : 0u;
                    }
                    bits(R, base, m);
                }
            }
        }
        A.add(R);
        if (FEAT) fs.cnt += R.hits;
    }
    if (REL)
        force_epilogue_rel<KAHAN, TENSION>(A, i, xi, ci, vi, ri, ph, g, map, F.collide, F.workIds, F.pos, F.vel,
                                           F.accS);
    else
        force_epilogue<KAHAN, TENSION, FEAT>(A, i, xi, vi, ri, ph, map, F.collide, F.workIds, F.pos, F.vel,
                                             F.accS, fs, F.fo);
}

// ---------------------------------------------------------------------------
// Force stage over reused neighbour lists: the pretested form over the rows
// the lists recorded (the density stage wrote this step's neighbour masks
// over them), then wall terms, integration, collision and write-back as
// k_force.  The next row's entries are loaded before the current row is
// walked.  It also records, for the decision at the next step, the largest
// squared distance of a particle from where it was when the lists were built.
// Occupancy: at most 56 registers, so nine 128-thread blocks fit on an SM
// (36 warps; at 64 registers eight): the single-scene forms spill 4-16
// bytes, the batched ones up to 88, and both run 1-2 % faster per step than
// at 64 registers without spills.  At 48 registers (ten blocks) the spills
// cost more than the warps gain.  A register cap, not a launch bound, so any
// block size the autotuner tries stays launchable.
// ---------------------------------------------------------------------------
// Displacement since the build into the scene's flag: one atomic per warp (or
// per scene a warp holds) that raises the recorded maximum.  Squared
// distances are non-negative, so their bits order as the values do; the
// maximum only grows, so a warp that does not exceed the value it reads
// (possibly an older, smaller one) has nothing to add.
template <bool BATCH>
__device__ __forceinline__ void record_displacement(const NeighbourLists& L, int scene, float d2) {
    const unsigned int v = __float_as_uint(d2);
    const unsigned int peers = BATCH ? __match_any_sync(0xffffffffu, scene) : 0xffffffffu;
    const unsigned int w = __reduce_max_sync(peers, v);
    unsigned int* f = L.flags + VL_DISP * L.numScenes + scene;
    if ((threadIdx.x & 31) == (unsigned int)(__ffs(peers) - 1) && w > 0u && w > *(volatile unsigned int*)f)
        atomicMax(f, w);
}

template <bool KAHAN, bool TENSION, bool BATCH>
__global__ void __maxnreg__(56)
k_force_lists(int n, const float4* __restrict__ posS, const float4* __restrict__ velS,
              const float4* __restrict__ rho4S, const int* __restrict__ workIds, PhysDev ph_, MapDev map_,
              int collideFlag, NeighbourLists L, float4* __restrict__ pos, float4* __restrict__ vel,
              float4* __restrict__ accS, const SceneDev* __restrict__ scenes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    int scene = 0;
    if (i < n) {
        const float4 xi = posS[i];
        const float4 vi = velS[i];
        const float4 ri = rho4S[i];
        if (BATCH) scene = L.slotScene[i];
        const PhysDev& ph = BATCH ? scenes[scene].ph : ph_;
        const MapDev& map = BATCH ? scenes[scene].map : map_;
        const float h2 = ph.h2;
        ForceTotals<KAHAN, TENSION> A;
        const int rows = L.rows[i];
        int svN = __ldg(L.start + i);
        uint2 mN = __ldg(L.exact + i);
        // a neighbour's p/rho^2 and 1/rho ride in the fourth lanes of its
        // sorted position and velocity (written by the density stage)
        auto pairs = [&](RowSums<TENSION>& R, int base, unsigned int m) {
            R.hits += __popc(m);
            while (m) {
                const int t = base + __ffs(m) - 1;
                m &= m - 1u;
                const float4 xj = __ldg(posS + t), vj = __ldg(velS + t);
                R.template add<false>(ph, Pair(ph, xi, vi, xj, vj), ri.z, make_float4(0.f, 0.f, xj.w, vj.w));
            }
        };
#pragma unroll 1
        for (int r = 0; r < rows; r++) {
            const int sv = svN;
            const uint2 m = mN;
            if (r + 1 < rows) {
                svN = __ldg(L.start + (size_t)(r + 1) * n + i);
                mN = __ldg(L.exact + (size_t)(r + 1) * n + i);
            }
            RowSums<TENSION> R;
            R.clear();
            if (sv < 0) {
                for (int t = sv & 0x7fffffff; t < (int)m.x; t++) {
                    const float4 xj = __ldg(posS + t);
                    if (neighbour_r2(dist2(xi, xj), h2)) {
                        const float4 vj = __ldg(velS + t);
                        R.add(ph, Pair(ph, xi, vi, xj, vj), ri.z, make_float4(0.f, 0.f, xj.w, vj.w));
                    }
                }
            } else {
                pairs(R, sv, m.x);
                pairs(R, sv + 32, m.y);
            }
            A.add(R);
        }
        float mapDist = 1e30f, mapN[3] = {0.f, 0.f, 0.f};
        float3 x, v;
        float acc[3];
        force_finish<KAHAN, TENSION, false>(A, xi, vi, ri, ph, map, collideFlag, x, v, acc, mapDist, mapN, xi);
        const int id = workIds[i];
        // (the sorted copy's fourth lane holds p/rho^2; a batch keeps the scene there)
        pos[id] = make_float4(x.x, x.y, x.z, BATCH ? __int_as_float(scene) : 0.f);
        vel[id] = make_float4(v.x, v.y, v.z, 0.f);
        accS[i] = make_float4(acc[0], acc[1], acc[2], 0.f);
        const float4 b = __ldg(L.posB + i);
        const float dx = x.x - b.x, dy = x.y - b.y, dz = x.z - b.z;
        d2 = dx * dx + dy * dy + dz * dz;
        if (!(d2 == d2)) d2 = __uint_as_float(0x7f800000u);  // NaN: as far as it gets
    }
    record_displacement<BATCH>(L, scene, d2);
}

// ---------------------------------------------------------------------------
// The pretested force form with each warp's neighbour rows staged in shared
// memory by TMA (plain handles).  The 32 particles of a warp are consecutive
// in the working order, so their windows into one stencil row overlap: the
// warp takes the union of its lanes' windows and one lane copies it into
// shared memory with three bulk copies (sorted position, velocity and
// density records, cp.async.bulk completing on an mbarrier).  Rows are
// double-buffered: row r + 1's copies are issued before row r is processed.
// Every lane then reads its neighbours from shared memory instead of
// gathering them through L1.  A row whose union exceeds ST_ROW candidates (a
// warp across a cell-row boundary, or a window too long for a mask) is read
// from global memory as before.  The same pairs in the same order: results
// are bit-identical to the other forms.  Each wait is bounded; a wait that
// gives up latches STATUS_DEVICE_WAIT, the warp reads global memory from
// then on and waits once more, bounded, for its copies still in flight.
// ---------------------------------------------------------------------------
constexpr int ST_ROW = 72;     // staged candidates per warp, row and buffer
constexpr int ST_WARPS = 8;    // 256-thread blocks
constexpr int ST_SMEM = ST_WARPS * 2 * 3 * ST_ROW * 16 + ST_WARPS * 2 * 8;
constexpr uint32_t ST_WAIT_LIMIT = 1u << 22;

template <bool KAHAN, bool TENSION>
__global__ void __launch_bounds__(ST_WARPS * 32, 4) k_force_staged(ForceArgs F, unsigned int* status) {
    extern __shared__ __align__(128) unsigned char stsm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* buf = reinterpret_cast<float4*>(stsm) + warp * (2 * 3 * ST_ROW);  // [buffer][P, V, Q][ST_ROW]
    uint64_t* bars = reinterpret_cast<uint64_t*>(stsm + ST_WARPS * 2 * 3 * ST_ROW * 16) + 2 * warp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < F.n;  // no early return: the warp stages its rows together
    if (lane == 0) {
        tc::mbar_init(bars, 1);
        tc::mbar_init(bars + 1, 1);
    }
    __syncwarp();
    float4 xi = make_float4(0.f, 0.f, 0.f, 0.f), vi = xi, ri = xi;
    if (valid) {
        xi = F.posS[i];
        vi = F.velS[i];
        ri = F.rho4S[i];
    }
    const PhysDev& ph = F.ph;
    ForceTotals<KAHAN, TENSION> A;
    // a row: this lane's window (start, mask) and the warp's staged union [u0, u0 + len)
    auto row_info = [&](int r, int& sv, unsigned int& mk, int& u0, int& len) {
        sv = 0;
        mk = 0u;
        int lo = INT_MAX, hi = INT_MIN;
        if (valid) {
            sv = __ldg(F.M.start + (size_t)r * F.n + i);
            mk = __ldg(F.M.mask + (size_t)r * F.n + i);
            if (sv >= 0 && mk) {
                lo = sv + __ffs(mk) - 1;
                hi = sv + 32 - __clz(mk);
            }
        }
        u0 = __reduce_min_sync(0xffffffffu, lo);
        const int u1 = __reduce_max_sync(0xffffffffu, hi);
        len = u1 > u0 ? u1 - u0 : 0;
        if (len > ST_ROW) len = -1;  // not staged
    };
    unsigned int phase = 0u, pending = 0u;  // per buffer: wait parity, copy in flight
    bool broken = false;
    auto issue = [&](int b, int u0, int len) {
        if (lane == 0) {
            float4* d = buf + b * 3 * ST_ROW;
            const uint32_t bytes = (uint32_t)len * 16u;
            tc::fence_async_smem();  // this warp's reads of the buffer come first
            tc::mbar_arrive_expect_tx(bars + b, 3u * bytes);
            tc::bulk_g2s(d, F.posS + u0, bytes, bars + b);
            tc::bulk_g2s(d + ST_ROW, F.velS + u0, bytes, bars + b);
            tc::bulk_g2s(d + 2 * ST_ROW, F.rho4S + u0, bytes, bars + b);
        }
        pending |= 1u << b;
    };
    int sv, u0, len;
    unsigned int mk;
    row_info(0, sv, mk, u0, len);
    if (len > 0) issue(0, u0, len);
#pragma unroll 1
    for (int r = 0; r < 9; r++) {
        const int b = r & 1;
        int svN = 0, u0N = 0, lenN = 0;
        unsigned int mkN = 0u;
        if (r + 1 < 9) {
            row_info(r + 1, svN, mkN, u0N, lenN);
            if (lenN > 0 && !broken) issue(b ^ 1, u0N, lenN);
        }
        bool staged = len > 0 && (pending >> b & 1u);
        if (staged) {
            const bool ok = __all_sync(0xffffffffu, tc::mbar_wait(bars + b, phase >> b & 1u, ST_WAIT_LIMIT));
            if (ok) {
                phase ^= 1u << b;
                pending &= ~(1u << b);
            } else {
                if (lane == 0 && status) atomicOr(status, STATUS_DEVICE_WAIT);
                broken = true;
                staged = false;
            }
        }
        RowSums<TENSION> R;
        R.clear();
        if (valid) {
            if (sv < 0) {
                // a window too long for a mask: test and interact from global memory
                for (int t = sv & 0x7fffffff; t < (int)mk; t++) {
                    const float4 xj = __ldg(F.posS + t);
                    const float r2 = dist2(xi, xj);
                    if (neighbour_r2(r2, ph.h2)) {
                        const float4 vj = __ldg(F.velS + t), rj = __ldg(F.rho4S + t);
                        R.add(ph, Pair(ph, xi, vi, xj, vj), ri.z, rj);
                    }
                }
            } else {
                const float4* P = buf + b * 3 * ST_ROW;
                R.hits += __popc(mk);
                while (mk) {
                    const int t = sv + __ffs(mk) - 1;
                    mk &= mk - 1u;
                    float4 xj, vj, rj;
                    if (staged) {
                        xj = P[t - u0];
                        vj = P[ST_ROW + t - u0];
                        rj = P[2 * ST_ROW + t - u0];
                    } else {
                        xj = __ldg(F.posS + t);
                        vj = __ldg(F.velS + t);
                        rj = __ldg(F.rho4S + t);
                    }
                    R.template add<false>(ph, Pair(ph, xi, vi, xj, vj), ri.z, rj);
                }
            }
        }
        __syncwarp();  // the buffer is refilled two rows on
        A.add(R);
        sv = svN;
        mk = mkN;
        u0 = u0N;
        len = lenN;
    }
    if (broken && lane == 0)  // copies still in flight land before the block leaves
        for (int b = 0; b < 2; b++)
            if (pending >> b & 1u) tc::mbar_wait(bars + b, phase >> b & 1u, ST_WAIT_LIMIT);
    __syncwarp();
    if (valid) {
        FeatSums fs;
        force_epilogue<KAHAN, TENSION, false>(A, i, xi, vi, ri, ph, F.map, F.collide, F.workIds, F.pos, F.vel,
                                              F.accS, fs, F.fo);
    }
}

// ---------------------------------------------------------------------------
// The learned step's force stage with the corrector fused in.  The pretested
// pair loop, wall terms, integration and collision of k_force, then the
// 24 features of each particle go straight to shared memory as a BF16 MMA
// operand.  The block's two 128-particle tiles run the MLP together: each
// layer is two tcgen05.mma groups (one per tile, accumulators in TMEM
// columns 64 * tile) behind one commit, and every warp then reads its own
// tile's accumulator lanes.  Each particle's correction is added before its
// single write-back.  Three or four blocks share an SM, so one block's MMA
// round trips overlap the others' pair loops.  The raw features also go to
// `fo.feat` when it is set.
// ---------------------------------------------------------------------------
// Shared memory is kept small: the pair loop's neighbour gathers live on
// the L1 cache, which shares the SM's 256 KB with it.  The operand region
// holds the two feature tiles until layer 1's MMAs have read them, then the
// two hidden tiles of layer 1, then those of layer 2.
constexpr int L_W = 0;                        // W1, W2, W3 (mlp::IMG_FWD_BYTES)
constexpr int L_X = mlp::IMG_FWD_BYTES;       // operand region: two 128 x 32 feature tiles, ...
constexpr int L_H = L_X;                      // ... later two 128 x 64 hidden tiles
constexpr int L_BIAS = L_H + 2 * 16384;
constexpr int L_NORM = L_BIAS + 4 * mlp::NBIAS;
constexpr int L_BAR = L_NORM + 4 * mlp::NNORM;  // MMA barrier, TMEM slot, weight-copy barrier
constexpr int L_SMEM = L_BAR + 32;
constexpr int L_TMEM = 128;                   // 4 blocks x 128 = 512 columns
constexpr int L_THREADS = 256;
// Resident blocks per SM: four (64 registers, a few spilled) when the grid
// fills the GPU several times over, the pair loop being latency bound; three
// (80 registers, no spills) for small grids, where per-thread latency counts.
constexpr int L_BLOCKS_MAX = 4;
static_assert(L_X % 1024 == 0 && L_BIAS % 16 == 0 && L_NORM % 16 == 0 && L_BAR % 8 == 0, "layout");
static_assert(L_BLOCKS_MAX * (L_SMEM + 1024) <= 227 * 1024 && L_BLOCKS_MAX * L_TMEM <= 512,
              "resident blocks per SM");

// LISTS: the neighbours come from the reused lists' exact masks (as in
// k_force_lists: the same pairs in the same order as the masks of the
// per-step search at a building step, the neighbours' p/rho^2 and 1/rho from
// the fourth lanes of their sorted position and velocity), and the kernel
// records the largest squared distance of a corrected position from where
// the particle was when the lists were built.
template <bool KAHAN, bool TENSION, int BLOCKS, bool LISTS>
__global__ void __launch_bounds__(L_THREADS, BLOCKS)
k_force_learned(ForceArgs F, MlpDev m, unsigned int* status, NeighbourLists L) {
    using namespace mlp;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ int sOk;
    const int t = threadIdx.x, warp = t >> 5, half = t >> 7, r = t & 127;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L_BAR);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + L_BAR + 8);
    uint64_t* wbar = reinterpret_cast<uint64_t*>(sm + L_BAR + 16);
    float* sBias = reinterpret_cast<float*>(sm + L_BIAS);
    float* sNorm = reinterpret_cast<float*>(sm + L_NORM);
    for (int k = t; k < NBIAS; k += L_THREADS) sBias[k] = epilogue_bias(m.bias, k);
    for (int k = t; k < NNORM; k += L_THREADS) sNorm[k] = m.norm[k];
    if (t == 0) {
        tc::mbar_init(bar, 1);
        tc::mbar_init(wbar, 1);
        sOk = 1;
        // the weight image arrives by one TMA bulk copy while the pair loop runs
        tc::mbar_arrive_expect_tx(wbar, IMG_FWD_BYTES);
        tc::bulk_g2s(sm + L_W, m.image, IMG_FWD_BYTES, wbar);
    }
    if (warp == 0) tc::tmem_alloc(slot, L_TMEM);
    tc::cta_sync();
    const uint32_t tb = *slot;
    const int i = blockIdx.x * L_THREADS + t;
    const bool valid = i < F.n;
    float3 x = make_float3(0.f, 0.f, 0.f), v = x;
    float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
    int id = 0;
    {
        float f[IN];
        if (valid) {
            xi = F.posS[i];
            const float4 vi = F.velS[i];
            const float4 ri = F.rho4S[i];
            const PhysDev& ph = F.ph;
            ForceTotals<KAHAN, TENSION> A;
            FeatSums fs;
            if (LISTS) {
                const int rows = L.rows[i];
#pragma unroll 1
                for (int row = 0; row < rows; row++) {
                    RowSums<TENSION> R;
                    R.clear();
                    const int sv = __ldg(L.start + (size_t)row * F.n + i);
                    const uint2 mk = __ldg(L.exact + (size_t)row * F.n + i);
                    if (sv < 0) {
                        for (int tt = sv & 0x7fffffff; tt < (int)mk.x; tt++) {
                            const float4 xj = __ldg(F.posS + tt);
                            if (neighbour_r2(dist2(xi, xj), ph.h2)) {
                                const float4 vj = __ldg(F.velS + tt), rj = make_float4(0.f, 0.f, xj.w, vj.w);
                                const Pair p(ph, xi, vi, xj, vj);
                                R.add(ph, p, ri.z, rj);
                                fs.add(ph, p, rj);
                            }
                        }
                    } else {
                        R.hits += __popc(mk.x) + __popc(mk.y);
#pragma unroll
                        for (int w = 0; w < 2; w++) {
                            unsigned int b = w ? mk.y : mk.x;
                            while (b) {
                                const int tt = sv + 32 * w + __ffs(b) - 1;
                                b &= b - 1u;
                                const float4 xj = __ldg(F.posS + tt), vj = __ldg(F.velS + tt);
                                const float4 rj = make_float4(0.f, 0.f, xj.w, vj.w);
                                const Pair p(ph, xi, vi, xj, vj);
                                R.template add<false>(ph, p, ri.z, rj);
                                fs.add(ph, p, rj);
                            }
                        }
                    }
                    A.add(R);
                    fs.cnt += R.hits;
                }
            }
#pragma unroll
            for (int row = 0; row < (LISTS ? 0 : 9); row++) {
                RowSums<TENSION> R;
                R.clear();
                const int sv = __ldg(F.M.start + (size_t)row * F.n + i);
                unsigned int mk = __ldg(F.M.mask + (size_t)row * F.n + i);
                if (sv < 0) {
                    for (int tt = sv & 0x7fffffff; tt < (int)mk; tt++) {
                        const float4 xj = __ldg(F.posS + tt);
                        const float r2 = dist2(xi, xj);
                        if (neighbour_r2(r2, ph.h2)) {
                            const float4 vj = __ldg(F.velS + tt), rj = __ldg(F.rho4S + tt);
                            const Pair p(ph, xi, vi, xj, vj);
                            R.add(ph, p, ri.z, rj);
                            fs.add(ph, p, rj);
                        }
                    }
                } else {
                    R.hits += __popc(mk);
                    while (mk) {
                        const int tt = sv + __ffs(mk) - 1;
                        mk &= mk - 1u;
                        const float4 xj = __ldg(F.posS + tt), vj = __ldg(F.velS + tt), rj = __ldg(F.rho4S + tt);
                        const Pair p(ph, xi, vi, xj, vj);
                        R.template add<false>(ph, p, ri.z, rj);
                        fs.add(ph, p, rj);
                    }
                }
                A.add(R);
                fs.cnt += R.hits;
            }
            float acc[3], mapDist = 1e30f, mapN[3] = {0.f, 0.f, 0.f};
            force_finish<KAHAN, TENSION, true>(A, xi, vi, ri, ph, F.map, F.collide, x, v, acc, mapDist, mapN, xi);
            id = F.workIds[i];
            F.accS[i] = make_float4(acc[0], acc[1], acc[2], 0.f);
            feature_values(fs, F.fo.boxWalls, F.fo.dtL, xi, vi, ri, acc, mapDist, mapN, ph, f);
            if (F.fo.feat) store_features(F.fo.feat, (size_t)(F.fo.byId ? id : i), f);
        }
        store_feature_row(sm + L_X + half * 8192, r, f, valid, sNorm);
    }
    const uint32_t sW = tc::smem_u32(sm + L_W);
    const uint32_t sX = tc::smem_u32(sm + L_X), sH = tc::smem_u32(sm + L_H);
    unsigned char* myH = sm + L_H + half * 16384;
    const uint32_t tl = tc::tmem_at(tb, 32 * (warp & 3), 64 * half);  // this warp's lanes of its tile
    uint32_t phase = 0;
    // sOk: 1 running, 0 an MMA wait gave up, 2 the weight copy never landed
    if (t == 0 && !tc::mbar_wait(wbar, 0, WAIT_LIMIT)) {
        sOk = 2;
        atomicOr(status, STATUS_DEVICE_WAIT);
    }
    tc::cta_sync();
    if (sOk == 1) do {
        tc::cta_sync();
        if (t == 0) {
            tc::mma_chain(tb, sX, sW + IMG_W1, INP, HID, false);
            tc::mma_chain(tb + 64, sX + 8192, sW + IMG_W1, INP, HID, false);
        }
        if (!commit_and_wait(bar, phase, &sOk, t)) break;
        hidden_layer_out(tl, sBias, myH, r);
        tc::cta_sync();
        if (t == 0) {
            tc::mma_chain(tb, sH, sW + IMG_W2, HID, HID, false);
            tc::mma_chain(tb + 64, sH + 16384, sW + IMG_W2, HID, HID, false);
        }
        // once the wait returns the MMAs have read layer 1's tiles: layer 2
        // overwrites them
        if (!commit_and_wait(bar, phase, &sOk, t)) break;
        hidden_layer_out(tl, sBias + HID, myH, r);
        tc::cta_sync();
        if (t == 0) {
            tc::mma_chain(tb, sH, sW + IMG_W3, HID, OUTP, false);
            tc::mma_chain(tb + 64, sH + 16384, sW + IMG_W3, HID, OUTP, false);
        }
        if (!commit_and_wait(bar, phase, &sOk, t)) break;
        float y[16];
        tc::tmem_ld16(tl, y);
        if (valid) {
            float c[OUT];
            decode_correction(sNorm, sBias + 2 * HID, y, c);
            x = make_float3(x.x + c[0], x.y + c[1], x.z + c[2]);
            v = make_float3(v.x + c[3], v.y + c[4], v.z + c[5]);
            if (F.collide) collide(F.ph, x, v);
            F.pos[id] = make_float4(x.x, x.y, x.z, LISTS ? 0.f : xi.w);
            F.vel[id] = make_float4(v.x, v.y, v.z, 0.f);
        }
    } while (false);
    tc::cta_sync();
    if (sOk == 0) drain(bar, phase, t, status);
    if (sOk == 2 && t == 0) tc::mbar_wait(wbar, 0, WAIT_LIMIT);  // once more for the copy in flight
    tc::cta_sync();
    if (warp == 0) tc::tmem_dealloc(tb, L_TMEM);
    if (LISTS) {  // as in k_force_lists
        float d2 = 0.f;
        if (valid) {
            const float4 b = __ldg(L.posB + i);
            const float dx = x.x - b.x, dy = x.y - b.y, dz = x.z - b.z;
            d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 == d2)) d2 = __uint_as_float(0x7f800000u);
        }
        record_displacement<false>(L, 0, d2);
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
void launch_density(int n, const float4* posS, RowTables T, GridDev g, PhysDev ph, MapDev map, float4* rho4S,
                    int* rowStart, unsigned int* rowMask, const StepConfig& cfg, cudaStream_t s) {
    if (n <= 0) return;
    const int bs = cfg.densityBlock > 0 ? cfg.densityBlock : 128;
    const int grid = (n + bs - 1) / bs;
    const RowMasks M{rowStart, rowMask};
    const bool emit = cfg.forceVariant >= FORCE_PRETESTED;  // the pretested and staged forms read masks
#define SPH_DENSITY(K, E, B) k_density<K, E, B, false><<<grid, bs, 0, s>>>(n, posS, T, g, ph, map, cfg.prune, rho4S, M)
#define SPH_DENSITY_REL(K, E) k_density<K, E, false, true><<<grid, bs, 0, s>>>(n, posS, T, g, ph, map, cfg.prune, rho4S, M)
    if (g.rel) {
        if (cfg.kahan) {
            if (emit) SPH_DENSITY_REL(true, true);
            else SPH_DENSITY_REL(true, false);
        } else {
            if (emit) SPH_DENSITY_REL(false, true);
            else SPH_DENSITY_REL(false, false);
        }
    } else if (T.scenes) {
        if (cfg.kahan) {
            if (emit) SPH_DENSITY(true, true, true);
            else SPH_DENSITY(true, false, true);
        } else {
            if (emit) SPH_DENSITY(false, true, true);
            else SPH_DENSITY(false, false, true);
        }
    } else {
        if (cfg.kahan) {
            if (emit) SPH_DENSITY(true, true, false);
            else SPH_DENSITY(true, false, false);
        } else {
            if (emit) SPH_DENSITY(false, true, false);
            else SPH_DENSITY(false, false, false);
        }
    }
#undef SPH_DENSITY
#undef SPH_DENSITY_REL
}

template <bool KAHAN, bool TENSION>
static void force_dispatch(const ForceArgs& F, const StepConfig& cfg, unsigned int* status, cudaStream_t s) {
    const int bs = cfg.forceBlock > 0 ? cfg.forceBlock : 128;
    const int grid = (F.n + bs - 1) / bs;
    if (F.T.scenes) {
        // batched scenes (plain steps only; no feature recording); the staged
        // form is the plain handles' only, the pretested one serves here
        if (cfg.forceVariant >= FORCE_PRETESTED)
            k_force<KAHAN, TENSION, FORCE_PRETESTED, false, true><<<grid, bs, 0, s>>>(F);
        else if (cfg.forceVariant == FORCE_MASK)
            k_force<KAHAN, TENSION, FORCE_MASK, false, true><<<grid, bs, 0, s>>>(F);
        else
            k_force<KAHAN, TENSION, FORCE_DIRECT, false, true><<<grid, bs, 0, s>>>(F);
    } else if (F.g.rel) {
        // cell-relative positions (plain steps only; the pretested form stands
        // in for the staged one)
        if (cfg.forceVariant >= FORCE_PRETESTED)
            k_force<KAHAN, TENSION, FORCE_PRETESTED, false, false, true><<<grid, bs, 0, s>>>(F);
        else if (cfg.forceVariant == FORCE_MASK)
            k_force<KAHAN, TENSION, FORCE_MASK, false, false, true><<<grid, bs, 0, s>>>(F);
        else
            k_force<KAHAN, TENSION, FORCE_DIRECT, false, false, true><<<grid, bs, 0, s>>>(F);
    } else if (F.fo.feat) {
        // the learned step's force stage records the corrector's features; the
        // density stage has recorded the neighbour masks (pretested form)
        k_force<KAHAN, TENSION, FORCE_PRETESTED, true, false><<<grid, bs, 0, s>>>(F);
    } else if (cfg.forceVariant == FORCE_STAGED) {
        ensure_dynamic_smem<k_force_staged<KAHAN, TENSION>>(ST_SMEM);
        k_force_staged<KAHAN, TENSION>
            <<<(F.n + ST_WARPS * 32 - 1) / (ST_WARPS * 32), ST_WARPS * 32, ST_SMEM, s>>>(F, status);
    } else if (cfg.forceVariant == FORCE_PRETESTED) {
        k_force<KAHAN, TENSION, FORCE_PRETESTED, false, false><<<grid, bs, 0, s>>>(F);
    } else if (cfg.forceVariant == FORCE_MASK) {
        k_force<KAHAN, TENSION, FORCE_MASK, false, false><<<grid, bs, 0, s>>>(F);
    } else {
        k_force<KAHAN, TENSION, FORCE_DIRECT, false, false><<<grid, bs, 0, s>>>(F);
    }
}

void launch_force(int n, const float4* posS, const float4* velS, const float4* rho4S, const int* workIds,
                  RowTables T, GridDev g, PhysDev ph, MapDev map, int collide, const int* rowStart,
                  const unsigned int* rowMask, float4* pos, float4* vel, float4* accS, const StepConfig& cfg,
                  cudaStream_t s, const FeatureOut* feat, unsigned int* status) {
    if (n <= 0) return;
    FeatOut fo{nullptr, 0, 0, 0.f};
    if (feat) fo = FeatOut{feat->feat, feat->byId, feat->boxWalls, feat->dtL};
    ForceArgs F{n,  posS, velS, rho4S, workIds, T, g, ph, map, collide, cfg.prune,
                RowMasks{const_cast<int*>(rowStart), const_cast<unsigned int*>(rowMask)}, pos, vel, accS, fo};
    const bool tension = ph.tension != 0.0f;
    if (cfg.kahan) {
        if (tension) force_dispatch<true, true>(F, cfg, status, s);
        else force_dispatch<true, false>(F, cfg, status, s);
    } else {
        if (tension) force_dispatch<false, true>(F, cfg, status, s);
        else force_dispatch<false, false>(F, cfg, status, s);
    }
}

template <bool KAHAN, bool TENSION, int BLOCKS, bool LISTS>
static void force_learned_launch(const ForceArgs& F, MlpDev m, unsigned int* status, const NeighbourLists& L,
                                 cudaStream_t s) {
    ensure_dynamic_smem<k_force_learned<KAHAN, TENSION, BLOCKS, LISTS>>(L_SMEM);
    k_force_learned<KAHAN, TENSION, BLOCKS, LISTS>
        <<<(F.n + L_THREADS - 1) / L_THREADS, L_THREADS, L_SMEM, s>>>(F, m, status, L);
}

template <bool KAHAN, bool TENSION, bool LISTS>
static void force_learned_dispatch(const ForceArgs& F, MlpDev m, unsigned int* status, const NeighbourLists& L,
                                   cudaStream_t s) {
    const int sms = device_sms();
    const long long blocks = (F.n + L_THREADS - 1) / L_THREADS;
    if (blocks >= 2LL * L_BLOCKS_MAX * sms)
        force_learned_launch<KAHAN, TENSION, L_BLOCKS_MAX, LISTS>(F, m, status, L, s);
    else
        force_learned_launch<KAHAN, TENSION, 3, LISTS>(F, m, status, L, s);
}

void launch_force_learned(int n, const float4* posS, const float4* velS, const float4* rho4S, const int* workIds,
                          RowTables T, GridDev g, PhysDev ph, MapDev map, int collide, const int* rowStart,
                          const unsigned int* rowMask, float4* pos, float4* vel, float4* accS, const StepConfig& cfg,
                          const FeatureOut& feat, MlpDev m, unsigned int* status, cudaStream_t s,
                          const NeighbourLists* lists) {
    if (n <= 0) return;
    const FeatOut fo{feat.feat, feat.byId, feat.boxWalls, feat.dtL};
    ForceArgs F{n,  posS, velS, rho4S, workIds, T, g, ph, map, collide, cfg.prune,
                RowMasks{const_cast<int*>(rowStart), const_cast<unsigned int*>(rowMask)}, pos, vel, accS, fo};
    const NeighbourLists L = lists ? *lists : NeighbourLists{};
    const bool tension = ph.tension != 0.0f;
#define SPH_FORCE_LEARNED(K, T)                                        \
    do {                                                               \
        if (lists) force_learned_dispatch<K, T, true>(F, m, status, L, s); \
        else force_learned_dispatch<K, T, false>(F, m, status, L, s);      \
    } while (0)
    if (cfg.kahan) {
        if (tension) SPH_FORCE_LEARNED(true, true);
        else SPH_FORCE_LEARNED(true, false);
    } else {
        if (tension) SPH_FORCE_LEARNED(false, true);
        else SPH_FORCE_LEARNED(false, false);
    }
#undef SPH_FORCE_LEARNED
}

// After the positions were written: the largest squared distance of a
// particle from where it was when the lists were built, in place of the one
// the steps accumulated (the next step builds the lists again only if that
// exceeds the rebuild distance).  flags[VL_DISP] must be zero on entry.
template <bool BATCH>
__global__ void k_list_displacement(int n, const float4* __restrict__ pos, const int* __restrict__ workIds,
                                    NeighbourLists L) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    int scene = 0;
    if (k < n) {
        const float4 x = __ldg(pos + workIds[k]), b = __ldg(L.posB + k);
        if (BATCH) scene = L.slotScene[k];
        const float dx = x.x - b.x, dy = x.y - b.y, dz = x.z - b.z;
        d2 = dx * dx + dy * dy + dz * dz;
        if (!(d2 == d2)) d2 = __uint_as_float(0x7f800000u);
    }
    record_displacement<BATCH>(L, scene, d2);
}

void launch_list_displacement(int n, const float4* pos, const int* workIds, const NeighbourLists& L, cudaStream_t s) {
    if (n <= 0) return;
    cudaMemsetAsync(L.flags + VL_DISP * L.numScenes, 0, sizeof(unsigned int) * L.numScenes, s);
    if (L.numScenes > 1) k_list_displacement<true><<<(n + 255) / 256, 256, 0, s>>>(n, pos, workIds, L);
    else k_list_displacement<false><<<(n + 255) / 256, 256, 0, s>>>(n, pos, workIds, L);
}

void launch_density_lists(int n, float4* posS, float4* velS, RowTables T, GridDev g, PhysDev ph, MapDev map,
                          float4* rho4S, const NeighbourLists& L, const StepConfig& cfg, bool build, bool reuse,
                          cudaStream_t s) {
    if (n <= 0) return;
    const int bs = cfg.densityBlock > 0 ? cfg.densityBlock : 128;
    const int grid = (n + bs - 1) / bs;
    const bool batch = T.scenes != nullptr;
#define SPH_DENSITY_BUILD(K, B) k_density_build<K, B><<<grid, bs, 0, s>>>(n, posS, velS, T, g, ph, map, rho4S, L)
#define SPH_DENSITY_LISTS(K, B) \
    k_density_lists<K, B><<<grid, bs, 0, s>>>(n, posS, velS, ph, map, rho4S, L, T.scenes)
    if (build) {
        if (cfg.kahan) {
            if (batch) SPH_DENSITY_BUILD(true, true);
            else SPH_DENSITY_BUILD(true, false);
        } else {
            if (batch) SPH_DENSITY_BUILD(false, true);
            else SPH_DENSITY_BUILD(false, false);
        }
    }
    if (reuse) {
        if (cfg.kahan) {
            if (batch) SPH_DENSITY_LISTS(true, true);
            else SPH_DENSITY_LISTS(true, false);
        } else {
            if (batch) SPH_DENSITY_LISTS(false, true);
            else SPH_DENSITY_LISTS(false, false);
        }
    }
#undef SPH_DENSITY_BUILD
#undef SPH_DENSITY_LISTS
}

void launch_force_lists(int n, const float4* posS, const float4* velS, const float4* rho4S, const int* workIds,
                        PhysDev ph, MapDev map, int collide, const NeighbourLists& L, float4* pos, float4* vel,
                        float4* accS, const StepConfig& cfg, cudaStream_t s, const SceneDev* scenes) {
    if (n <= 0) return;
    const int bs = cfg.forceBlock > 0 ? cfg.forceBlock : 128;
    const int grid = (n + bs - 1) / bs;
    // (a batch's tension coefficient is the largest of its scenes': it selects
    // whether the colour field is computed at all)
    const bool tension = ph.tension != 0.0f;
#define SPH_FORCE_LISTS(K, T, B)                                                                             \
    k_force_lists<K, T, B><<<grid, bs, 0, s>>>(n, posS, velS, rho4S, workIds, ph, map, collide, L, pos, vel, \
                                               accS, scenes)
#define SPH_FORCE_LISTS_B(K, T)           \
    do {                                  \
        if (scenes) SPH_FORCE_LISTS(K, T, true);  \
        else SPH_FORCE_LISTS(K, T, false);        \
    } while (0)
    if (cfg.kahan) {
        if (tension) SPH_FORCE_LISTS_B(true, true);
        else SPH_FORCE_LISTS_B(true, false);
    } else {
        if (tension) SPH_FORCE_LISTS_B(false, true);
        else SPH_FORCE_LISTS_B(false, false);
    }
#undef SPH_FORCE_LISTS_B
#undef SPH_FORCE_LISTS
}

}  // namespace sph
