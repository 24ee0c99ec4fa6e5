// Boundary maps of "SPH in complex shapes" (SphInComplexShapes.cpp:203-427),
// built on the GPU.
//
// The reference scatters each ghost particle's poly6 / viscosity-kernel value
// onto the grid nodes within its support (SetBox, :269-304).  Here every node
// gathers from the ghost lattice points within its support instead, visiting
// them in the same k, j, i lattice order the reference creates its ghosts in,
// so each node's sum is accumulated in the reference's order and needs no
// atomics.  This file is compiled with --fmad=false: node positions, signed
// distances and kernel values are formed one rounded operation at a time, as
// the reference's host code does.
#include <math.h>

#include "sph_internal.h"

namespace sph {
namespace {

struct MapArgs {
    float start[3];
    float spacing;
    unsigned int dims[3];
    float restDistance, h, mass, restDensity, viscosity, ps;
    int numShapes;
    sph_shape shapes[8];
    int boxOnly;             // one box container: SetBox's ghost rule
    int boxIndex;
    float latStart[3];       // ghost lattice origin and last index per axis
    unsigned int latMax[3];
    // SPH_SHAPE_MESH solids: the signed distance grid of shape slot i
    const float* grid[8];
    float gridOrigin[8][3];
    float gridDx[8];
    unsigned int gridDims[8][3];
};

// Trilinear signed distance of a grid solid (negative inside); no solid
// outside the grid's box.
__device__ double grid_sdf(const MapArgs& A, int s, const double* x) {
    double w[3];
    size_t i0[3];
    for (int a = 0; a < 3; a++) {
        const unsigned int n = A.gridDims[s][a];
        const double u = (x[a] - (double)A.gridOrigin[s][a]) / (double)A.gridDx[s];
        if (!(u >= 0.0) || u > (double)(n - 1)) return 1e30;
        const double f = n > 1 ? fmin(floor(u), (double)(n - 2)) : 0.0;
        i0[a] = (size_t)f;
        w[a] = n > 1 ? u - f : 0.0;
    }
    const unsigned int* d = A.gridDims[s];
    auto at = [&](int di, int dj, int dk) {
        const size_t ii = i0[0] + (d[0] > 1 ? di : 0), jj = i0[1] + (d[1] > 1 ? dj : 0),
                     kk = i0[2] + (d[2] > 1 ? dk : 0);
        return (double)A.grid[s][ii + (size_t)d[0] * (jj + (size_t)d[1] * kk)];
    };
    const double c00 = at(0, 0, 0) + w[0] * (at(1, 0, 0) - at(0, 0, 0));
    const double c10 = at(0, 1, 0) + w[0] * (at(1, 1, 0) - at(0, 1, 0));
    const double c01 = at(0, 0, 1) + w[0] * (at(1, 0, 1) - at(0, 0, 1));
    const double c11 = at(0, 1, 1) + w[0] * (at(1, 1, 1) - at(0, 1, 1));
    const double c0 = c00 + w[1] * (c10 - c00), c1 = c01 + w[1] * (c11 - c01);
    return c0 + w[2] * (c1 - c0);
}

// computeSignedDistancePoint3Box3 (SphInComplexShapes.cpp:714-747), axis-aligned.
__device__ float box_signed_distance(const float* pos, const float* c, const float* e) {
    float t[3] = {pos[0] - c[0], pos[1] - c[1], pos[2] - c[2]};
    float a = fabsf(t[0]) - e[0];
    float b = fabsf(t[1]) - e[1];
    float cc = fabsf(t[2]) - e[2];
    float distance = fabsf(a) < fabsf(b) ? a : b;
    if (fabsf(distance) > fabsf(cc)) distance = cc;
    if (a > 0.0f || b > 0.0f || cc > 0.0f) {
        float sq = 0.0f;
        for (int k = 0; k < 3; k++) {
            float d = 0.0f;
            if (t[k] < -e[k]) d = t[k] + e[k];
            else if (t[k] > e[k]) d = t[k] - e[k];
            sq += d * d;
        }
        distance = sqrtf(sq);
    }
    return distance;
}

__device__ bool inside_box(const float* pos, const float* c, const float* e) {
    for (int k = 0; k < 3; k++)
        if (fabsf(pos[k] - c[k]) >= e[k]) return false;
    return true;
}

// Solid cone on its base disc: distance to the triangle (0,0)-(R,0)-(0,H) in
// the (radial, axial) half-plane, negative inside.
__device__ double cone_sdf(const double* x, const float* p) {
    double q = sqrt((x[0] - p[0]) * (x[0] - p[0]) + (x[1] - p[1]) * (x[1] - p[1]));
    double z = x[2] - p[2];
    double R = p[3], H = p[4];
    double bq = fmin(fmax(q, 0.0), R);
    double d2 = (q - bq) * (q - bq) + z * z;
    double ex = -R, ez = H;
    double t = ((q - R) * ex + z * ez) / (ex * ex + ez * ez);
    t = fmin(fmax(t, 0.0), 1.0);
    double sx = q - (R + t * ex), sz = z - t * ez;
    d2 = fmin(d2, sx * sx + sz * sz);
    bool inside = z >= 0.0 && z <= H && q <= R * (1.0 - z / H);
    double d = sqrt(d2);
    return inside ? -d : d;
}

// Distance to the solid, positive in the fluid.
__device__ float solid_distance(const MapArgs& A, const float* xf) {
    double x[3] = {xf[0], xf[1], xf[2]};
    double s = 1e30;
    for (int i = 0; i < A.numShapes; i++) {
        const sph_shape& S = A.shapes[i];
        double d;
        if (S.kind == SPH_SHAPE_SPHERE) {
            double dx = x[0] - S.p[0], dy = x[1] - S.p[1], dz = x[2] - S.p[2];
            d = sqrt(dx * dx + dy * dy + dz * dz) - S.p[3];
        } else if (S.kind == SPH_SHAPE_CONE) {
            d = cone_sdf(x, S.p);
        } else if (S.kind == SPH_SHAPE_MESH) {
            d = grid_sdf(A, i, x);
        } else {
            d = -(double)box_signed_distance(xf, S.p, S.p + 3);
        }
        s = fmin(s, d);
    }
    return (float)s;
}

// evaluateDensityKernel / evaluateViscosityKernel (SphInComplexShapes.cpp:666-690).
__device__ float eval_density_kernel(float sqDist, float h) {
    float coeff = (float)(315.0f / (64.0f * 3.14159265358979323846 * h * h * h * h * h * h * h * h * h));
    float sqh = h * h;
    float diff = sqh - sqDist;
    if (diff < 0.0f) return 0.0f;
    return coeff * diff * diff * diff;
}

__device__ float eval_viscosity_kernel(float sqDist, float h) {
    float dist = sqrtf(sqDist);
    if (dist > h) return 0.0f;
    return (float)(45.0f / (3.14159265358979323846 * h * h * h * h * h * h) * (h - dist));
}

__device__ void node_pos(const MapArgs& A, int i, int j, int k, float* p) {
    p[0] = A.start[0] + A.spacing * (float)i;
    p[1] = A.start[1] + A.spacing * (float)j;
    p[2] = A.start[2] + A.spacing * (float)k;
}

__global__ void k_build_maps(MapArgs A, float* dist, float* dens, float* visc, float4* map4) {
    size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)A.dims[0] * A.dims[1] * A.dims[2];
    if (n >= total) return;
    int i = (int)(n % A.dims[0]);
    int j = (int)((n / A.dims[0]) % A.dims[1]);
    int k = (int)(n / ((size_t)A.dims[0] * A.dims[1]));
    float np[3];
    node_pos(A, i, j, k, np);
    float d = -solid_distance(A, np);
    float outD = -A.restDistance, outRho = 0.0f, outVis = 0.0f;
    if (fabsf(d) < A.h) {
        if (fabsf(d) > A.restDistance) d = d / fabsf(d) * A.restDistance;
        outD = d;
        // ghost lattice points that can lie within h of this node
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            float f0 = floorf((np[a] - A.h - A.latStart[a]) / A.ps) - 1.0f;
            float f1 = floorf((np[a] + A.h - A.latStart[a]) / A.ps) + 1.0f;
            f0 = fmaxf(f0, 0.0f);
            f1 = fminf(f1, (float)A.latMax[a]);
            lo[a] = (int)f0;
            hi[a] = (int)f1;
        }
        const sph_shape& B = A.shapes[A.boxIndex];
        for (int kk = lo[2]; kk <= hi[2]; kk++)
            for (int jj = lo[1]; jj <= hi[1]; jj++)
                for (int ii = lo[0]; ii <= hi[0]; ii++) {
                    float g[3] = {A.latStart[0] + (float)ii * A.ps, A.latStart[1] + (float)jj * A.ps,
                                  A.latStart[2] + (float)kk * A.ps};
                    bool ghost = A.boxOnly ? !inside_box(g, B.p, B.p + 3)
                                           : solid_distance(A, g) <= 0.0f;
                    if (!ghost) continue;
                    float dx = g[0] - np[0], dy = g[1] - np[1], dz = g[2] - np[2];
                    float sq = dx * dx + dy * dy + dz * dz;
                    outRho += eval_density_kernel(sq, A.h);
                    outVis += eval_viscosity_kernel(sq, A.h);
                }
        outRho *= A.mass;
        outVis *= A.viscosity * A.mass / A.restDensity;
    }
    if (dist) dist[n] = outD;
    if (dens) dens[n] = outRho;
    if (visc) visc[n] = outVis;
    if (map4) map4[n] = make_float4(outD, outRho, outVis, 0.0f);
}

}  // namespace

cudaError_t launch_build_maps(const sph_boundary_desc& D, const unsigned int dims[3], float* dist, float* dens,
                              float* visc, float4* map4, cudaStream_t s) {
    MapArgs A{};
    for (int a = 0; a < 3; a++) {
        A.start[a] = D.gridStart[a];
        A.dims[a] = dims[a];
    }
    A.spacing = D.gridSpacing;
    A.restDistance = D.restDistance;
    A.h = D.compactSupport;
    A.mass = D.particleMass;
    A.restDensity = D.restDensity;
    A.viscosity = D.viscosity;
    A.ps = D.particleSpacing;
    A.numShapes = D.numShapes;
    A.boxIndex = 0;
    int boxes = 0;
    for (int i = 0; i < D.numShapes && i < 8; i++) {
        A.shapes[i] = D.shapes[i];
        if (D.shapes[i].kind == SPH_SHAPE_BOX) {
            if (boxes == 0) A.boxIndex = i;
            boxes++;
        }
    }
    A.boxOnly = (boxes == 1 && D.numShapes == 1) ? 1 : 0;
    // Ghost lattice: SetBox's (SphInComplexShapes.cpp:233-244) around a box
    // container, else the map grid grown by compactSupport + particleSpacing.
    float margin = D.compactSupport + D.particleSpacing;
    for (int a = 0; a < 3; a++) {
        if (boxes > 0) {
            const sph_shape& B = D.shapes[A.boxIndex];
            float ext = B.p[3 + a] + margin;
            A.latStart[a] = B.p[a] - ext;
            A.latMax[a] = (unsigned int)(2 * ext / D.particleSpacing);
        } else {
            float len = (float)(dims[a] - 1) * D.gridSpacing + 2 * margin;
            A.latStart[a] = D.gridStart[a] - margin;
            A.latMax[a] = (unsigned int)(len / D.particleSpacing);
        }
    }
    size_t total = (size_t)dims[0] * dims[1] * dims[2];
    if (total == 0) return cudaSuccess;
    // grid solids: device copies of their distances for the build
    float* devGrid[8] = {};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < D.numShapes && i < 8 && e == cudaSuccess; i++) {
        if (D.shapes[i].kind != SPH_SHAPE_MESH) continue;
        const sph_sdf_grid& G = D.sdfGrids[(int)D.shapes[i].p[0]];
        const size_t nodes = (size_t)G.dims[0] * G.dims[1] * G.dims[2];
        e = cudaMalloc((void**)&devGrid[i], sizeof(float) * nodes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(devGrid[i], G.distance, sizeof(float) * nodes, cudaMemcpyHostToDevice, s);
        A.grid[i] = devGrid[i];
        A.gridDx[i] = G.dx;
        for (int a = 0; a < 3; a++) {
            A.gridOrigin[i][a] = G.origin[a];
            A.gridDims[i][a] = G.dims[a];
        }
    }
    if (e == cudaSuccess) {
        k_build_maps<<<(unsigned int)((total + 127) / 128), 128, 0, s>>>(A, dist, dens, visc, map4);
        e = cudaGetLastError();
    }
    bool any = false;
    for (float* g : devGrid) any = any || g;
    if (any) {
        const cudaError_t w = cudaStreamSynchronize(s);  // the grids are freed after the build
        if (e == cudaSuccess) e = w;
        for (float* g : devGrid)
            if (g) cudaFree(g);
    }
    return e;
}

}  // namespace sph
