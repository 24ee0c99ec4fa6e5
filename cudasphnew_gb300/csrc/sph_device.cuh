// Device helpers shared by the step kernels: the reference's grid arithmetic
// (bit-exact), the software trilinear boundary-map fetch, neighbour-row
// iteration over the 27-cell stencil, compensated summation and the box
// collision response.
#pragma once

#include "sph_internal.h"

namespace sph {

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
    return g.cellBase + h;
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
        int lo = (int)f;  // saturating conversion; clamped below
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

__device__ __forceinline__ size_t map_node(const MapDev& m, int x, int y, int z) {
    return (size_t)x + (size_t)m.dims[0] * ((size_t)y + (size_t)m.dims[1] * (size_t)z);
}

__device__ __forceinline__ float tri_scalar(const MapDev& m, const float* __restrict__ g, float u,
                                            float v, float w) {
    Tri t = tri_setup(m, u, v, w);
    float c00 = lerp_ref(__ldg(g + map_node(m, t.i0[0], t.i0[1], t.i0[2])),
                         __ldg(g + map_node(m, t.i1[0], t.i0[1], t.i0[2])), t.a[0]);
    float c10 = lerp_ref(__ldg(g + map_node(m, t.i0[0], t.i1[1], t.i0[2])),
                         __ldg(g + map_node(m, t.i1[0], t.i1[1], t.i0[2])), t.a[0]);
    float c01 = lerp_ref(__ldg(g + map_node(m, t.i0[0], t.i0[1], t.i1[2])),
                         __ldg(g + map_node(m, t.i1[0], t.i0[1], t.i1[2])), t.a[0]);
    float c11 = lerp_ref(__ldg(g + map_node(m, t.i0[0], t.i1[1], t.i1[2])),
                         __ldg(g + map_node(m, t.i1[0], t.i1[1], t.i1[2])), t.a[0]);
    return lerp_ref(lerp_ref(c00, c10, t.a[1]), lerp_ref(c01, c11, t.a[1]), t.a[2]);
}

__device__ __forceinline__ float4 lerp4(float4 p, float4 q, float a) {
    return make_float4(lerp_ref(p.x, q.x, a), lerp_ref(p.y, q.y, a), lerp_ref(p.z, q.z, a), 0.f);
}

// (distance, wall density, wall viscosity) at one point, from the
// interleaved float4 map: one pass over the 8 corner nodes.
__device__ __forceinline__ float4 tri_vec(const MapDev& m, float u, float v, float w) {
    Tri t = tri_setup(m, u, v, w);
    const float4* g = m.map4;
    float4 c00 = lerp4(__ldg(g + map_node(m, t.i0[0], t.i0[1], t.i0[2])),
                       __ldg(g + map_node(m, t.i1[0], t.i0[1], t.i0[2])), t.a[0]);
    float4 c10 = lerp4(__ldg(g + map_node(m, t.i0[0], t.i1[1], t.i0[2])),
                       __ldg(g + map_node(m, t.i1[0], t.i1[1], t.i0[2])), t.a[0]);
    float4 c01 = lerp4(__ldg(g + map_node(m, t.i0[0], t.i0[1], t.i1[2])),
                       __ldg(g + map_node(m, t.i1[0], t.i0[1], t.i1[2])), t.a[0]);
    float4 c11 = lerp4(__ldg(g + map_node(m, t.i0[0], t.i1[1], t.i1[2])),
                       __ldg(g + map_node(m, t.i1[0], t.i1[1], t.i1[2])), t.a[0]);
    return lerp4(lerp4(c00, c10, t.a[1]), lerp4(c01, c11, t.a[1]), t.a[2]);
}

// u = (pos - origin)/gridLength (particle_simulation.cu:243-245).
__device__ __forceinline__ void map_uvw(const MapDev& m, float4 x, float* uvw) {
    uvw[0] = __fdiv_rn(__fsub_rn(x.x, m.origin[0]), m.length[0]);
    uvw[1] = __fdiv_rn(__fsub_rn(x.y, m.origin[1]), m.length[1]);
    uvw[2] = __fdiv_rn(__fsub_rn(x.z, m.origin[2]), m.length[2]);
}

// ---------------------------------------------------------------------------
// Neighbour rows: the 3x3 (z, y) rows of the 27-cell stencil
// (particle_simulation.cu:225-238).  Cells of one row are consecutive hashes,
// so the candidates of a row are one contiguous range [s, e) of the sorted
// arrays, visited in the reference's k, j, i order.
//
// With `window`, a row whose (y, z) cell rectangle lies farther than h from
// the particle is skipped, and the others are cut to the half-cells (in x)
// that the sphere of radius h reaches at that (y, z) gap: the working order
// sorts each cell by x and records where its upper half starts, so the cut
// is a table lookup.  The gap is shrunk and the reach grown by 1e-3 h -- far
// more than the rounding of any cell boundary or distance -- so every particle
// within h stays a candidate; the candidates dropped all lie beyond h and
// contribute exactly nothing in the reference either.
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

__device__ __forceinline__ float cell_gap(float p, int c, float origin, float spacing, float eps) {
    float lo = origin + (float)c * spacing;
    float hi = lo + spacing;
    return fmaxf(fmaxf(lo - p, p - hi) - eps, 0.0f);
}

// Squared distance with every rounding spelled out, so the density stage
// (which records neighbour masks) and the force stage (which uses them or
// tests again) decide each pair identically.
__device__ __forceinline__ float dist2(float4 a, float4 b) {
    const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// A pair interacts when 0 < r^2 <= h^2.  r^2 is a sum of squares (or NaN),
// so its bits order as the values do: one integer compare.
__device__ __forceinline__ bool neighbour_r2(float r2, float h2) {
    return __float_as_uint(r2) - 1u < __float_as_uint(h2);
}

// Candidate range [s, e) of stencil row r (0..8: k outer, j inner).  Rows
// outside the stencil and rows the window cut removes are empty (s == e).
__device__ __forceinline__ void row_range(float4 xi, const Stencil& st, float h, const GridDev& g, RowTables T,
                                          bool window, int r, int& s, int& e) {
    s = e = 0;
    const int z = st.z0 + r / 3, y = st.y0 + r % 3;
    if (z > st.z1 || y > st.y1) return;
    const int row = g.cellBase + g.dim[0] * (g.dim[1] * z + y);
    if (!window) {
        s = __ldg(T.cellOffset + row + st.x0);
        e = __ldg(T.cellOffset + row + st.x1 + 1);
        return;
    }
    const float eps = 1e-3f * h;
    const float h2 = h * h;
    const float gz = cell_gap(xi.z, z, g.origin[2], g.spacing, eps);
    const float gy = cell_gap(xi.y, y, g.origin[1], g.spacing, eps);
    const float g2 = gy * gy + gz * gz;
    if (g2 > h2) return;
    const float inv = 1.0f / g.spacing;
    // the reach in x: an approximate square root (relative error ~2^-22) is
    // far inside the eps margin
    float rx;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(rx) : "f"(h2 - g2));
    rx += eps;
    const float xl = xi.x - rx, xr = xi.x + rx;
    const int cl = max(st.x0, (int)floorf((xl - g.origin[0]) * inv));
    const int cr = min(st.x1, (int)floorf((xr - g.origin[0]) * inv));
    if (cl > cr) return;
    const int a0 = __ldg(T.cellOffset + row + cl), a1 = __ldg(T.cellOffset + row + cl + 1);
    const int b0 = __ldg(T.cellOffset + row + cr), b1 = __ldg(T.cellOffset + row + cr + 1);
    const float midL = g.origin[0] + ((float)cl + 0.5f) * g.spacing;
    const float midR = g.origin[0] + ((float)cr + 0.5f) * g.spacing;
    s = a0;
    e = b1;
    if (xl >= midL) s = min(max(__ldg(T.halfOffset + row + cl), a0), a1);
    if (xr < midR) e = min(max(__ldg(T.halfOffset + row + cr), b0), b1);
    if (e < s) e = s;
}

// Candidate window [s, e) of the grid row (y, z) for a sphere of radius R
// around xi: the row is skipped when its (y, z) cell rectangle lies farther
// than R, and otherwise cut to the half-cells in x that the sphere reaches at
// that gap, clamped to the grid (not to the 27-cell stencil: R may exceed a
// cell).  The same margins as row_range, so every particle within R is a
// candidate.  Used to build the reused neighbour lists.
__device__ __forceinline__ bool row_window(float4 xi, int y, int z, float R, float eps, const GridDev& g,
                                           RowTables T, int& s, int& e) {
    s = e = 0;
    const float R2 = R * R;
    const float gz = cell_gap(xi.z, z, g.origin[2], g.spacing, eps);
    const float gy = cell_gap(xi.y, y, g.origin[1], g.spacing, eps);
    const float g2 = gy * gy + gz * gz;
    if (g2 > R2) return false;
    const float inv = 1.0f / g.spacing;
    float rx;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(rx) : "f"(R2 - g2));
    rx += eps;
    const float xl = xi.x - rx, xr = xi.x + rx;
    const int cl = max(0, (int)floorf((xl - g.origin[0]) * inv));
    const int cr = min(g.dim[0] - 1, (int)floorf((xr - g.origin[0]) * inv));
    if (cl > cr) return false;
    const int row = g.cellBase + g.dim[0] * (g.dim[1] * z + y);
    const int a0 = __ldg(T.cellOffset + row + cl), a1 = __ldg(T.cellOffset + row + cl + 1);
    const int b0 = __ldg(T.cellOffset + row + cr), b1 = __ldg(T.cellOffset + row + cr + 1);
    const float midL = g.origin[0] + ((float)cl + 0.5f) * g.spacing;
    const float midR = g.origin[0] + ((float)cr + 0.5f) * g.spacing;
    s = a0;
    e = b1;
    if (xl >= midL) s = min(max(__ldg(T.halfOffset + row + cl), a0), a1);
    if (xr < midR) e = min(max(__ldg(T.halfOffset + row + cr), b0), b1);
    if (e < s) e = s;
    return e > s;
}

// The cell range [lo, hi] of axis `a` that [p - r, p + r] touches, clamped to the grid.
__device__ __forceinline__ void cell_span(float p, float r, const GridDev& g, int a, int& lo, int& hi) {
    const float inv = 1.0f / g.spacing;
    lo = max(0, (int)floorf((p - r - g.origin[a]) * inv));
    hi = min(g.dim[a] - 1, (int)floorf((p + r - g.origin[a]) * inv));
}

// ---------------------------------------------------------------------------
// Cell-relative positions (sph_options.cellRelative): .xyz is the offset from
// the low corner of the particle's cell, .w carries the cell's integer
// coordinates packed 11:11:10 bits (x lowest).  A neighbour in a cell dc
// cells away sits at rel_j + dc * spacing in i's frame; every pair offset is
// then a difference of numbers no larger than two cells, whatever the
// distance from the grid origin.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int3 rel_cell(float4 p) {
    const unsigned int u = __float_as_uint(p.w);
    return make_int3((int)(u & 0x7ffu), (int)((u >> 11) & 0x7ffu), (int)(u >> 22));
}

__device__ __forceinline__ float rel_pack(int cx, int cy, int cz) {
    return __uint_as_float((unsigned int)cx | ((unsigned int)cy << 11) | ((unsigned int)cz << 22));
}

__device__ __forceinline__ int rel_cx(float w) { return (int)(__float_as_uint(w) & 0x7ffu); }

// The absolute FP32 position origin + c * spacing + rel, summed in FP64 and
// rounded once (for the boundary maps, the wall box and read-back): a
// position converted in with rel_from_abs comes back bit for bit.
__device__ __forceinline__ float4 rel_abs(float4 p, int3 c, const GridDev& g) {
    const double s = (double)g.spacing;
    return make_float4((float)((double)g.origin[0] + (double)c.x * s + (double)p.x),
                       (float)((double)g.origin[1] + (double)c.y * s + (double)p.y),
                       (float)((double)g.origin[2] + (double)c.z * s + (double)p.z), 0.f);
}

// Neighbour j (cell-relative, in its own cell) in i's frame: y and z cell
// offsets are those of the stencil row (dyo, dzo already times spacing), the
// x offset is read from j's packed cell.
__device__ __forceinline__ float4 rel_in_frame(float4 pj, int cxi, float dyo, float dzo, float spacing) {
    return make_float4(fmaf((float)(rel_cx(pj.w) - cxi), spacing, pj.x), pj.y + dyo, pj.z + dzo, 0.f);
}

// An absolute position's cell (the reference hash's coordinates, clamped to
// the grid) and its offset from that cell's low corner, formed in FP64 so the
// offset is the FP32 position's own, correctly rounded.
__device__ __forceinline__ void rel_from_abs(float3 xa, const GridDev& g, float3& rel, int3& c) {
    const float v[3] = {xa.x, xa.y, xa.z};
    float o[3];
    int cc[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float f = __fdiv_rn(__fsub_rn(v[a], g.origin[a]), g.spacing);
        int k = isfinite(f) ? (int)f : 0;
        k = k % g.dim[a];
        k = min(max(k, 0), g.dim[a] - 1);
        cc[a] = k;
        o[a] = (float)((double)v[a] - ((double)g.origin[a] + (double)k * (double)g.spacing));
    }
    rel = make_float3(o[0], o[1], o[2]);
    c = make_int3(cc[0], cc[1], cc[2]);
}

// The stencil of a cell-relative particle: the neighbour cells its sphere of
// radius h <= spacing can reach, clamped to the grid.
__device__ __forceinline__ Stencil stencil_rel(float4 x, int3 c, float h, const GridDev& g) {
    Stencil s;
    s.x0 = x.x - h < 0.f ? max(c.x - 1, 0) : c.x;
    s.x1 = x.x + h >= g.spacing ? min(c.x + 1, g.dim[0] - 1) : c.x;
    s.y0 = x.y - h < 0.f ? max(c.y - 1, 0) : c.y;
    s.y1 = x.y + h >= g.spacing ? min(c.y + 1, g.dim[1] - 1) : c.y;
    s.z0 = x.z - h < 0.f ? max(c.z - 1, 0) : c.z;
    s.z1 = x.z + h >= g.spacing ? min(c.z + 1, g.dim[2] - 1) : c.z;
    return s;
}

// row_range for a cell-relative particle: the same rows and half-cell cut,
// with every boundary taken in the particle's own cell frame.  Also returns
// the row's y and z offsets (times spacing) for rel_in_frame.
__device__ __forceinline__ void row_range_rel(float4 xi, int3 c, const Stencil& st, float h, const GridDev& g,
                                              RowTables T, bool window, int r, int& s, int& e, float& dyo,
                                              float& dzo) {
    s = e = 0;
    const int z = st.z0 + r / 3, y = st.y0 + r % 3;
    dyo = (float)(y - c.y) * g.spacing;
    dzo = (float)(z - c.z) * g.spacing;
    if (z > st.z1 || y > st.y1) return;
    const int row = g.cellBase + g.dim[0] * (g.dim[1] * z + y);
    if (!window) {
        s = __ldg(T.cellOffset + row + st.x0);
        e = __ldg(T.cellOffset + row + st.x1 + 1);
        return;
    }
    const float eps = 1e-3f * h;
    const float h2 = h * h;
    const float gz = cell_gap(xi.z, 0, dzo, g.spacing, eps);
    const float gy = cell_gap(xi.y, 0, dyo, g.spacing, eps);
    const float g2 = gy * gy + gz * gz;
    if (g2 > h2) return;
    const float inv = 1.0f / g.spacing;
    // the reach in x: an approximate square root (relative error ~2^-22) is
    // far inside the eps margin
    float rx;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(rx) : "f"(h2 - g2));
    rx += eps;
    const float xl = xi.x - rx, xr = xi.x + rx;
    const int cl = max(st.x0, c.x + (int)floorf(xl * inv));
    const int cr = min(st.x1, c.x + (int)floorf(xr * inv));
    if (cl > cr) return;
    const int a0 = __ldg(T.cellOffset + row + cl), a1 = __ldg(T.cellOffset + row + cl + 1);
    const int b0 = __ldg(T.cellOffset + row + cr), b1 = __ldg(T.cellOffset + row + cr + 1);
    const float midL = ((float)(cl - c.x) + 0.5f) * g.spacing;
    const float midR = ((float)(cr - c.x) + 0.5f) * g.spacing;
    s = a0;
    e = b1;
    if (xl >= midL) s = min(max(__ldg(T.halfOffset + row + cl), a0), a1);
    if (xr < midR) e = min(max(__ldg(T.halfOffset + row + cr), b0), b1);
    if (e < s) e = s;
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float term) {
    float y = __fsub_rn(term, comp);
    float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

// collision_handling (particle_simulation.cu:742-834) for one particle, with
// two guards the reference lacks (it yields NaN there): |v| == 0 drops the
// restitution term, and a contact point that rounds onto the particle leaves
// it untouched.
// `cen` is the box centre in the frame x is given in (the absolute
// ph.boxCen, or the centre relative to a cell corner for cell-relative
// positions).
__device__ __forceinline__ void collide_box(const float* cen, const PhysDev& ph, float3& x, float3& v) {
    float lx = x.x - cen[0], ly = x.y - cen[1], lz = x.z - cen[2];
    float dist = fmaxf(fmaxf(fabsf(lx) - ph.boxDim[0], fabsf(ly) - ph.boxDim[1]),
                       fabsf(lz) - ph.boxDim[2]);
    if (!(dist > 0.f)) return;
    float cx = fminf(ph.boxDim[0], fmaxf(-ph.boxDim[0], lx)) + cen[0];
    float cy = fminf(ph.boxDim[1], fmaxf(-ph.boxDim[1], ly)) + cen[1];
    float cz = fminf(ph.boxDim[2], fmaxf(-ph.boxDim[2], lz)) + cen[2];
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

__device__ __forceinline__ void collide(const PhysDev& ph, float3& x, float3& v) { collide_box(ph.boxCen, ph, x, v); }

}  // namespace sph
