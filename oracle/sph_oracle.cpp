// =============================================================================
//  sph_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
//  CPU restatement of the CUDASPHNEW SPH step, used as the parity checker for
//  the GB300 library and as the timed CPU baseline.  Nothing in the product
//  (the cudasphnew_gb300 package, its shared library or the public headers)
//  links, loads or calls this file; only the tests, __graft_entry__.smoke()
//  and bench.py's CPU-baseline / reference legs do.
//
//  Every function is templated on the arithmetic type R:
//    R = float  : the reference's FP32 operation order ("ref32"), used for the
//                 bit-exact integer outputs (hash, permutation, cell table) and
//                 as the timed CPU baseline;
//    R = double : the same formulas in FP64 ("oracle64"), used as the yardstick for
//                 densities, pressures and accelerations, together with the
//                 per-particle magnitude scales the tolerances are quoted on.
//
//  The reference cannot be compiled here (Windows/GL headers, CUDA texture
//  references that CUDA 12+ removed, missing WildMagic5 binaries), so parity is
//  anchored on this restatement; the boundary maps are pinned against the
//  reference's own recorded output images distances.ppm / viscosities.ppm.
//  Citations are CUDASPHNEW/<file>:<line>.
//
//  Build: oracle/build_oracle.sh (g++ -O2 -fopenmp -ffp-contract=off).
//  -ffp-contract=off matters: the reference's FP32 expressions are evaluated
//  one rounded operation at a time, and aarch64 gcc would otherwise fuse them.
// =============================================================================
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Byte-identical to struct SimulationParameters, particle_simulation.h:54-111.
struct OrcParams {
    float gridOrigin[3];
    float gridSpacing;
    int gridDim[3];
    float gridSpacingSubParticles;
    int gridDimSubParticles[3];
    unsigned int numParticles;
    float compactSupport;
    float compactSupportSub;
    int kernelParticles;
    float timeStep;
    float timeStepSubParticles;
    float particleMass;
    float subParticleMass;
    float gasStiffness;
    float restDensity;
    float dynamicViscosity;
    float gravity;
    float tensionCoefficient;
    float normThresh;
    float fluidVolume;
    float poly6, gradPoly6, laplPoly6, gradSpiky, laplVisc;
    float poly6Sub, gradPoly6Sub, laplPoly6Sub, gradSpikySub, laplViscSub;
    float cmDistanceThresh;
    float nPartTresh;
    float boxDim[3];
    float boxCen[3];
    float restitution;
};

// Options that the reference hard-codes.  Mirrors sph_options in
// include/sph.h field for field (the tests fill both from one ctypes struct).
struct OrcOptions {
    int gravityAxis;      // reference: 1 (acc.y -= gravity, particle_simulation.cu:471)
    int boxCollision;     // run collision_handling after integrate (AdvanceTwoScale order)
    int childMode;        // 0: children re-seeded every step; 1: persistent + merge-back
    int reserved1;
    float splitMin[3];    // two-scale split region (reference: 0.2 <= x <= 0.5)
    float splitMax[3];
};

// Boundary maps as dense x-fastest float grids (CreateXTextureData layout,
// SphInComplexShapes.cpp:366-427) plus the texture metadata that
// setUpSphInComplexShapes uploads (particle_simulation.cu:2617-2642).
struct OrcMaps {
    float origin[3];
    float spacing;
    unsigned int dims[3];
    float restDistance;
    const float* dist;
    const float* dens;
    const float* visc;
};

}  // extern "C"

namespace {

const int EMPTY = -1;  // 0xFFFFFFFF, particle_simulation.cu:1661

int g_threads = 1;

// --------------------------------------------------------------------------
// Grid helpers
// --------------------------------------------------------------------------

// CUDA's float -> unsigned conversion (cvt.rzi.u32.f32) saturates: NaN and
// negative values give 0, values >= 2^32 give 0xFFFFFFFF.  The reference relies
// on this in compute_grid_coordinate (particle_simulation.cu:1242-1247).
template <class R>
unsigned int sat_u32(R f) {
    if (!(f > R(0))) return 0u;
    if (f >= R(4294967296.0)) return 0xFFFFFFFFu;
    return (unsigned int)f;
}

// compute_grid_coordinate / _sub_particles, particle_simulation.cu:1238-1284.
template <class R>
int grid_coord(R p, R d, R origin, R spacing, int dim) {
    unsigned int u = sat_u32<R>(((p + d) - origin) / spacing);
    int g = (int)u;
    g = g % dim;
    g = std::min(std::max(g, 0), dim - 1);
    return g;
}

// Hash of compute_particle_hash, particle_simulation.cu:100-115.  Returns
// false when the conversion would overflow an int (particle far outside).
template <class R>
bool particle_hash(const R* x, const float* origin, R spacing, const int* dim,
                   int* out) {
    int c[3];
    for (int a = 0; a < 3; a++) {
        R f = (x[a] - R(origin[a])) / spacing;
        if (!(std::fabs((double)f) < 2147483520.0)) return false;
        c[a] = (int)f;
        c[a] = c[a] % dim[a];
    }
    *out = dim[0] * (dim[1] * c[2] + c[1]) + c[0];
    return true;
}

// --------------------------------------------------------------------------
// tex3D emulation: normalised coordinates, linear filtering, clamp addressing
// (set_up_3d_float_texture, particle_simulation.cu:3003-3007).  Texel-space
// coordinate is u*N - 0.5 as for any CUDA normalised-coordinate fetch; the
// interpolation weights are exact (not the 9-bit fixed-point weights of the
// texture unit), matching the GPU library's software trilinear path.  Each
// linear blend is evaluated as v0 + a*(v1 - v0), which reproduces a constant
// field exactly: in the maps' clamped region (distance == -restDistance) the
// wall test distWall < restDistance must not fire on a rounding error.
// --------------------------------------------------------------------------
template <class R>
R tex3d(const float* g, const unsigned int* dims, R u, R v, R w) {
    R c[3] = {u * R(dims[0]) - R(0.5), v * R(dims[1]) - R(0.5),
              w * R(dims[2]) - R(0.5)};
    int i0[3], i1[3];
    R a[3];
    for (int k = 0; k < 3; k++) {
        R f = std::floor(c[k]);
        a[k] = c[k] - f;
        long long lo = (long long)f;
        long long hi = lo + 1;
        long long n = dims[k];
        i0[k] = (int)std::min(std::max(lo, 0LL), n - 1);
        i1[k] = (int)std::min(std::max(hi, 0LL), n - 1);
    }
    auto at = [&](int x, int y, int z) -> R {
        return R(g[(size_t)x + (size_t)dims[0] * ((size_t)y + (size_t)dims[1] * (size_t)z)]);
    };
    auto lerp = [](R v0, R v1, R t) -> R { return v0 + t * (v1 - v0); };
    R c00 = lerp(at(i0[0], i0[1], i0[2]), at(i1[0], i0[1], i0[2]), a[0]);
    R c10 = lerp(at(i0[0], i1[1], i0[2]), at(i1[0], i1[1], i0[2]), a[0]);
    R c01 = lerp(at(i0[0], i0[1], i1[2]), at(i1[0], i0[1], i1[2]), a[0]);
    R c11 = lerp(at(i0[0], i1[1], i1[2]), at(i1[0], i1[1], i1[2]), a[0]);
    return lerp(lerp(c00, c10, a[1]), lerp(c01, c11, a[1]), a[2]);
}

template <class R>
void map_uvw(const OrcMaps* M, const R* x, R* uvw) {
    for (int a = 0; a < 3; a++) {
        R len = R((float)(M->dims[a] - 1) * M->spacing);  // gridLength, :2628-2631
        uvw[a] = (x[a] - R(M->origin[a])) / len;
    }
}

// --------------------------------------------------------------------------
// Per-particle neighbourhood loop over the 27 cells in k, j, i order with the
// candidates of each cell in sorted order (particle_simulation.cu:225-238).
// --------------------------------------------------------------------------
template <class R, class F>
void for_each_cell(const OrcParams& P, const R* xi, R support, R spacing,
                   const int* dim, const int* start, const int* end, F&& f) {
    int c0[3], c1[3];
    for (int a = 0; a < 3; a++) {
        c0[a] = grid_coord<R>(xi[a], -support, R(P.gridOrigin[a]), spacing, dim[a]);
        c1[a] = grid_coord<R>(xi[a], support, R(P.gridOrigin[a]), spacing, dim[a]);
    }
    for (int k = c0[2]; k <= c1[2]; k++)
        for (int j = c0[1]; j <= c1[1]; j++)
            for (int i = c0[0]; i <= c1[0]; i++) {
                int h = dim[0] * (dim[1] * k + j) + i;
                f(start[h], end[h]);
            }
}

template <class R>
struct Level {
    R h, mass, poly6, grad, lapl, grad2, lapl2, spacing, dt;
    const int* dim;
};

template <class R>
Level<R> coarse_level(const OrcParams& P) {
    return Level<R>{R(P.compactSupport), R(P.particleMass), R(P.poly6), R(P.gradSpiky),
                    R(P.laplVisc), R(P.gradPoly6), R(P.laplPoly6), R(P.gridSpacing),
                    R(P.timeStep), P.gridDim};
}

template <class R>
Level<R> sub_level(const OrcParams& P) {
    return Level<R>{R(P.compactSupportSub), R(P.subParticleMass), R(P.poly6Sub),
                    R(P.gradSpikySub), R(P.laplViscSub), R(P.gradPoly6Sub),
                    R(P.laplPoly6Sub), R(P.gridSpacingSubParticles),
                    R(P.timeStepSubParticles), P.gridDimSubParticles};
}

// --------------------------------------------------------------------------
// Density + pressure: compute_particle_density_pressure (:196-256) with
// compute_particle_density_cell (:1385-1419).  Per-cell partial sums are
// added to the running total exactly as the reference does.  When `withWall`
// the wall density tex3D term is added (:242-248); the sub-particle kernel
// (:259-313) has no wall term.  `scale` (optional) receives the sum of the
// magnitudes of all terms (all positive here, so scale == rho).
// --------------------------------------------------------------------------
template <class R>
void density_one(const OrcParams& P, const Level<R>& L, const OrcMaps* M, bool withWall,
                 const R* pos, const int* ids, const int* start, const int* end,
                 const R* xi, R* rho, R* prs) {
    R density = R(0);
    R h = L.h;
    for_each_cell<R>(P, xi, h, L.spacing, L.dim, start, end, [&](int s, int e) {
        R cell = R(0);
        for (int u = s; u < e; u++) {
            const R* p = pos + 3 * (size_t)ids[u];
            R dx = p[0] - xi[0], dy = p[1] - xi[1], dz = p[2] - xi[2];
            R r = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (r <= h) {
                R d = h * h - r * r;
                cell += L.poly6 * d * d * d;
            }
        }
        density += cell;
    });
    density *= L.mass;
    if (withWall && M) {
        R uvw[3];
        map_uvw<R>(M, xi, uvw);
        density += tex3d<R>(M->dens, M->dims, uvw[0], uvw[1], uvw[2]);
    }
    *rho = density;
    *prs = R(P.gasStiffness) * (density - R(P.restDensity));
}

// --------------------------------------------------------------------------
// Acceleration: compute_particle_acceleration_ifsurf (:315-474) with
// compute_viscosity_pressure_forces_and_ifsurf_cell (:1459-1556), and the
// sub-particle variant compute_sub_particle_acceleration (:477-568) /
// compute_sub_particle_viscosity_pressure_forces_cell (:1558-1643) when
// `sub` is set (single force accumulator, no wall terms, tension always).
// colLapl starts at 0 (uninitialised in the reference, :381).
// `scale` receives the rounding-error scale of the FP32 evaluation: the sum of
// the magnitudes of every quantity that enters a sum or a difference, divided
// by rho, plus |g|.  A pressure p enters as k*(rho + rho0) (the magnitude that
// rounding of rho perturbs); the wall penalty coefficient
// rho/dt^2*(restDist - distWall) enters as rho/dt^2*(restDist + |distWall|) and
// each gradient component (t+ - t-)/(2 dX) as (|t+| + |t-|)/(2 dX).
// `scaleDirect` (optional) is the same sum with the wall terms taken at their
// own magnitude; it bounds differences between two evaluations that share the
// reference's operation order for the wall terms.
// --------------------------------------------------------------------------
template <class R>
void force_one(const OrcParams& P, const OrcOptions& O, const Level<R>& L,
               const OrcMaps* M, bool sub, const R* pos, const R* vel, const R* rhoA,
               const R* prsA, const int* ids, const int* start, const int* end,
               size_t i, R* acc, R* scale, R* scaleDirect = nullptr) {
    const R* xi = pos + 3 * i;
    const R* vi = vel + 3 * i;
    R rhoi = rhoA[i], pi = prsA[i];
    R h = L.h, grad = L.grad, lapl = L.lapl, grad2 = L.grad2, lapl2 = L.lapl2;
    R rhoi2 = rhoi * rhoi;
    R m = L.mass, mu = R(P.dynamicViscosity);
    R pF[3] = {0, 0, 0}, vF[3] = {0, 0, 0}, cg[3] = {0, 0, 0};
    R colLapl = R(0);
    double sc = 0.0;
    const double kS = (double)P.gasStiffness;
    const double rho0 = (double)P.restDensity;
    for_each_cell<R>(P, xi, h, L.spacing, L.dim, start, end, [&](int s, int e) {
        for (int u = s; u < e; u++) {
            size_t j = (size_t)ids[u];
            const R* xj = pos + 3 * j;
            const R* vj = vel + 3 * j;
            R rhoj = rhoA[j], pj = prsA[j];
            R r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
            R rn = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            R pressure = rhoi * (pi / rhoi2 + pj / (rhoj * rhoj)) * m;
            if (rn <= h && rn > R(0)) {
                R d = (h - rn) * (h - rn);
                for (int a = 0; a < 3; a++) pF[a] -= pressure * grad * d / rn * r[a];
                d = (h - rn);
                // the sub-particle kernel adds both into one force (:1619-1628)
                R* vacc = sub ? pF : vF;
                for (int a = 0; a < 3; a++) vacc[a] += mu * (vj[a] - vi[a]) * m / rhoj * lapl * d;
                d = (h * h - rn * rn) * (h * h - rn * rn);
                for (int a = 0; a < 3; a++) cg[a] += m / rhoj * grad2 * d * r[a];
                d = (h * h - rn * rn) * (R(3) * h * h - R(7) * rn * rn);
                colLapl += m / rhoj * lapl2 * d;
                if (scale) {
                    double hr = (double)h - (double)rn;
                    double Pi = kS * ((double)rhoi + rho0), Pj = kS * ((double)rhoj + rho0);
                    double mag = (double)rhoi * (Pi / ((double)rhoi * rhoi) +
                                                 Pj / ((double)rhoj * rhoj)) *
                                 (double)m * std::fabs((double)grad) * hr * hr;
                    double vmag = std::sqrt((double)vi[0] * vi[0] + (double)vi[1] * vi[1] +
                                            (double)vi[2] * vi[2]) +
                                  std::sqrt((double)vj[0] * vj[0] + (double)vj[1] * vj[1] +
                                            (double)vj[2] * vj[2]);
                    sc += mag + (double)mu * vmag * (double)m / (double)rhoj *
                                    std::fabs((double)lapl) * hr;
                }
            }
        }
    });

    R force[3];
    double wallScale = 0.0, wallDirect = 0.0, tensScale = 0.0;
    bool tension = true;
    if (!sub) {
        for (int a = 0; a < 3; a++) force[a] = R(0) + vF[a];
        for (int a = 0; a < 3; a++) force[a] += pF[a];
        if (M) {
            R uvw[3];
            map_uvw<R>(M, xi, uvw);
            R distWall = -tex3d<R>(M->dist, M->dims, uvw[0], uvw[1], uvw[2]);
            R rest = R(M->restDistance);
            R dt = R(P.timeStep);
            R coeff = rhoi / (dt * dt) * (rest - distWall);
            // within rounding of the band edge either branch is a correct
            // FP32 outcome: the scale then covers the wall term as well
            bool nearEdge = (double)distWall < (double)rest * (1.0 + 1e-5);
            if (distWall < rest || (scale && nearEdge)) {
                bool taken = distWall < rest;
                if (taken) tension = false;
                R dX[3], gN[3];
                double gAbs2 = 0.0;
                for (int a = 0; a < 3; a++)
                    dX[a] = R(M->spacing) / R((float)(M->dims[a] - 1) * M->spacing);
                R up[3], dn[3];
                for (int a = 0; a < 3; a++) {
                    for (int b = 0; b < 3; b++) {
                        up[b] = uvw[b];
                        dn[b] = uvw[b];
                    }
                    up[a] = uvw[a] + dX[a];
                    dn[a] = uvw[a] - dX[a];
                    R tp = tex3d<R>(M->dist, M->dims, up[0], up[1], up[2]);
                    R tm = tex3d<R>(M->dist, M->dims, dn[0], dn[1], dn[2]);
                    gN[a] = (tp - tm) / (R(2) * dX[a]);
                    double ga = (std::fabs((double)tp) + std::fabs((double)tm)) / (2.0 * (double)dX[a]);
                    gAbs2 += ga * ga;
                }
                R vw = tex3d<R>(M->visc, M->dims, uvw[0], uvw[1], uvw[2]);
                if (taken) {
                    for (int a = 0; a < 3; a++) force[a] -= coeff * gN[a];
                    for (int a = 0; a < 3; a++) force[a] -= vi[a] * vw;
                }
                if (scale) {
                    double gn = std::sqrt((double)gN[0] * gN[0] + (double)gN[1] * gN[1] +
                                          (double)gN[2] * gN[2]);
                    double vn = std::sqrt((double)vi[0] * vi[0] + (double)vi[1] * vi[1] +
                                          (double)vi[2] * vi[2]);
                    double cAbs = (double)rhoi / ((double)dt * (double)dt) *
                                  ((double)rest + std::fabs((double)distWall));
                    wallScale = cAbs * std::sqrt(gAbs2) + vn * std::fabs((double)vw);
                    wallDirect = std::fabs((double)coeff) * gn + vn * std::fabs((double)vw);
                }
            }
        }
    } else {
        for (int a = 0; a < 3; a++) force[a] = pF[a];
    }
    if (tension) {
        R colGraNorm = std::sqrt(cg[0] * cg[0] + cg[1] * cg[1] + cg[2] * cg[2]);
        R fCoeff = R(P.tensionCoefficient) * colLapl / colGraNorm;
        if (colGraNorm > R(P.normThresh)) {
            for (int a = 0; a < 3; a++) force[a] -= fCoeff * cg[a];
            if (scale) tensScale = std::fabs((double)fCoeff) * (double)colGraNorm;
        }
    }
    for (int a = 0; a < 3; a++) acc[a] = force[a] / rhoi;
    acc[O.gravityAxis] -= R(P.gravity);
    if (scale) {
        *scale = R((sc + wallScale + tensScale) / std::fabs((double)rhoi) +
                   std::fabs((double)P.gravity));
    }
    if (scaleDirect) {
        *scaleDirect = R((sc + wallDirect + tensScale) / std::fabs((double)rhoi) +
                         std::fabs((double)P.gravity));
    }
}

// --------------------------------------------------------------------------
// collision_handling (:742-834).  Two guards the reference lacks (it produces
// NaN there): |v| == 0 drops the restitution term instead of dividing by zero,
// and a contact point that rounds onto the particle (depth == 0) leaves the
// particle untouched.  `dt` is gSimParamsDev.timeStep for both levels.
// --------------------------------------------------------------------------
template <class R>
void collide_one(const OrcParams& P, R* x, R* v) {
    R local[3], diff[3];
    for (int a = 0; a < 3; a++) {
        local[a] = x[a] - R(P.boxCen[a]);
        diff[a] = std::fabs(local[a]) - R(P.boxDim[a]);
    }
    R dist = std::max(diff[0], diff[1]);
    dist = std::max(dist, diff[2]);
    if (!(dist > R(0))) return;
    R contact[3];
    for (int a = 0; a < 3; a++) {
        contact[a] = std::min(R(P.boxDim[a]), std::max(-R(P.boxDim[a]), local[a]));
        contact[a] += R(P.boxCen[a]);
    }
    R dd[3] = {contact[0] - x[0], contact[1] - x[1], contact[2] - x[2]};
    R depth = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
    if (!(depth > R(0))) return;
    R nrm[3] = {x[0] - contact[0], x[1] - contact[1], x[2] - contact[2]};
    R nn = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    for (int a = 0; a < 3; a++) nrm[a] /= nn;
    R velNorm = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    R dp = nrm[0] * v[0] + nrm[1] * v[1] + nrm[2] * v[2];
    R coeff;
    if (velNorm > R(0))
        coeff = (R(1) + R(P.restitution) * depth / (R(P.timeStep) * velNorm)) * dp;
    else
        coeff = dp;
    for (int a = 0; a < 3; a++) v[a] -= coeff * nrm[a];
    for (int a = 0; a < 3; a++) x[a] = contact[a];
}

// integrate_euler (:632-665): symplectic Euler, in place.
template <class R>
void integrate_one(R dt, const R* acc, R* x, R* v) {
    for (int a = 0; a < 3; a++) v[a] += dt * acc[a];
    for (int a = 0; a < 3; a++) x[a] += dt * v[a];
}

// Stable counting sort of (hash, id) by hash: the permutation that
// thrust::sort_by_key's stable radix sort produces (:2340-2343).
bool stable_sort_by_hash(int* hash, int* ids, int n, int numCells) {
    std::vector<int> cnt((size_t)numCells + 1, 0);
    for (int i = 0; i < n; i++) {
        if (hash[i] < 0 || hash[i] >= numCells) return false;
        cnt[(size_t)hash[i] + 1]++;
    }
    for (int c = 0; c < numCells; c++) cnt[(size_t)c + 1] += cnt[c];
    std::vector<int> h2(n), i2(n);
    for (int i = 0; i < n; i++) {
        int d = cnt[hash[i]]++;
        h2[d] = hash[i];
        i2[d] = ids[i];
    }
    std::memcpy(hash, h2.data(), sizeof(int) * (size_t)n);
    std::memcpy(ids, i2.data(), sizeof(int) * (size_t)n);
    return true;
}

// compute_cell_start_end (:155-193) after the two EMPTY memsets (:2362-2363).
void cell_start_end(const int* sortedHash, int n, int numCells, int* start, int* end) {
    std::fill(start, start + numCells, EMPTY);
    std::fill(end, end + numCells, EMPTY);
    for (int i = 0; i < n; i++) {
        int h = sortedHash[i];
        if (i == 0 || h != sortedHash[i - 1]) {
            start[h] = i;
            if (i > 0) end[sortedHash[i - 1]] = i;
        }
        if (i == n - 1) end[h] = i + 1;
    }
}

template <class R>
int hash_all(const OrcParams& P, const Level<R>& L, const R* pos, int n, int* hash,
             int* ids) {
    int bad = 0;
    for (int i = 0; i < n; i++) {
        if (!particle_hash<R>(pos + 3 * (size_t)i, P.gridOrigin, L.spacing, L.dim, &hash[i]))
            bad++;
        ids[i] = i;
    }
    return bad;
}

int num_cells(const int* dim) { return dim[0] * dim[1] * dim[2]; }

// The plain step: Advance (:2085-2117) without the two-scale bookkeeping,
// plus handleCollisions when O.boxCollision (AdvanceTwoScale, :2170).
template <class R>
int step_plain(const OrcParams& P, const OrcOptions& O, const OrcMaps* M, int n, R* pos,
               R* vel, R* rho, R* prs, R* acc, R* scaleRho, R* scaleAcc, R* scaleAccDirect,
               int* hash, int* ids, int* start, int* end) {
    Level<R> L = coarse_level<R>(P);
    int C = num_cells(P.gridDim);
    if (hash_all<R>(P, L, pos, n, hash, ids)) return 1;
    if (!stable_sort_by_hash(hash, ids, n, C)) return 2;
    cell_start_end(hash, n, C, start, end);
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
    for (int i = 0; i < n; i++) {
        density_one<R>(P, L, M, true, pos, ids, start, end, pos + 3 * (size_t)i, &rho[i],
                       &prs[i]);
        if (scaleRho) scaleRho[i] = rho[i];
    }
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
    for (int i = 0; i < n; i++)
        force_one<R>(P, O, L, M, false, pos, vel, rho, prs, ids, start, end, (size_t)i,
                     acc + 3 * (size_t)i, scaleAcc ? &scaleAcc[i] : nullptr,
                     scaleAccDirect ? &scaleAccDirect[i] : nullptr);
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < n; i++) {
        integrate_one<R>(R(P.timeStep), acc + 3 * (size_t)i, pos + 3 * (size_t)i,
                         vel + 3 * (size_t)i);
        if (O.boxCollision) collide_one<R>(P, pos + 3 * (size_t)i, vel + 3 * (size_t)i);
    }
    return 0;
}

}  // namespace

// =============================================================================
//  C entry points (ctypes)
// =============================================================================
extern "C" {

void orc_set_threads(int n) { g_threads = n > 0 ? n : 1; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// compute_particle_hash: returns the number of particles whose hash could not
// be formed (outside the representable range).
int orc_hash(const OrcParams* P, const float* pos, int n, int* hash, int* ids) {
    return hash_all<float>(*P, coarse_level<float>(*P), pos, n, hash, ids);
}

int orc_sort(int* hash, int* ids, int n, int numCells) {
    return stable_sort_by_hash(hash, ids, n, numCells) ? 0 : 1;
}

void orc_cells(const int* sortedHash, int n, int numCells, int* start, int* end) {
    cell_start_end(sortedHash, n, numCells, start, end);
}

// One plain step in FP32 (reference operation order); state updated in place.
int orc_step_plain_f32(const OrcParams* P, const OrcOptions* O, const OrcMaps* M, int n,
                       float* pos, float* vel, float* rho, float* prs, float* acc, int* hash,
                       int* ids, int* start, int* end) {
    return step_plain<float>(*P, *O, M, n, pos, vel, rho, prs, acc, nullptr, nullptr, nullptr,
                             hash, ids, start, end);
}

// The same step in FP64, with the tolerance scales.
int orc_step_plain_f64(const OrcParams* P, const OrcOptions* O, const OrcMaps* M, int n,
                       double* pos, double* vel, double* rho, double* prs, double* acc,
                       double* scaleRho, double* scaleAcc, double* scaleAccDirect, int* hash,
                       int* ids, int* start, int* end) {
    return step_plain<double>(*P, *O, M, n, pos, vel, rho, prs, acc, scaleRho, scaleAcc,
                              scaleAccDirect, hash, ids, start, end);
}

// Trilinear sample of one map at world positions (checks the emulated tex3D).
void orc_tex3d(const OrcMaps* M, int which, const double* xyz, int n, double* out) {
    const float* g = which == 0 ? M->dist : which == 1 ? M->dens : M->visc;
    for (int i = 0; i < n; i++) {
        double uvw[3];
        map_uvw<double>(M, xyz + 3 * (size_t)i, uvw);
        out[i] = tex3d<double>(g, M->dims, uvw[0], uvw[1], uvw[2]);
    }
}

}  // extern "C"

// =============================================================================
//  Boundary maps ("SPH in complex shapes", SphInComplexShapes.cpp)
// =============================================================================
extern "C" {

// One solid primitive.  kind 1: sphere obstacle (cx, cy, cz, r); kind 2: cone
// obstacle standing on its base disc (bx, by, bz, R, H), axis +z; kind 3: box
// container (cx, cy, cz, ex, ey, ez) whose INSIDE is fluid (SetBox's box).
struct OrcShape {
    int kind;
    float p[7];
};

// SphInComplexShapes(s, e, gridSpacing, restDistance, compactSupport,
// particleMass, restDensity, viscosity, particleSpacing)
// (SphInComplexShapes.cpp:34-64) plus the shapes handed to SetBox.
struct OrcBoundaryDesc {
    float gridStart[3];
    float gridEnd[3];
    float gridSpacing;
    float restDistance;
    float compactSupport;
    float particleMass;
    float restDensity;
    float viscosity;
    float particleSpacing;
    int numShapes;
    OrcShape shapes[8];
};

}  // extern "C"

namespace {

// computeSignedDistancePoint3Box3 (SphInComplexShapes.cpp:714-747) for an
// axis-aligned box.  The outside branch calls Wm5::DistPoint3Box3f::Get, whose
// implementation is only in a missing binary library: restated from geometry as
// the length of the per-axis excess outside the box, accumulated x, y, z.
float box_signed_distance(const float* pos, const float* c, const float* e) {
    float t[3] = {pos[0] - c[0], pos[1] - c[1], pos[2] - c[2]};
    float a = std::fabs(t[0]) - e[0];
    float b = std::fabs(t[1]) - e[1];
    float cc = std::fabs(t[2]) - e[2];
    float distance = std::fabs(a) < std::fabs(b) ? a : b;
    if (std::fabs(distance) > std::fabs(cc)) distance = cc;
    if (a > 0.0f || b > 0.0f || cc > 0.0f) {
        float sq = 0.0f;
        for (int k = 0; k < 3; k++) {
            float d = 0.0f;
            if (t[k] < -e[k]) d = t[k] + e[k];
            else if (t[k] > e[k]) d = t[k] - e[k];
            sq += d * d;
        }
        distance = std::sqrt(sq);
    }
    return distance;
}

// isInsideBox (SphInComplexShapes.cpp:699-712), axis-aligned.
bool inside_box(const float* pos, const float* c, const float* e) {
    for (int k = 0; k < 3; k++)
        if (std::fabs(pos[k] - c[k]) >= e[k]) return false;
    return true;
}

// Signed distance to a cone standing on its base disc (centre b, radius R,
// height H along +z), negative inside: distance in the (radial, axial)
// half-plane to the triangle (0,0)-(R,0)-(0,H).
double cone_sdf(const double* x, const float* p) {
    double q = std::sqrt((x[0] - p[0]) * (x[0] - p[0]) + (x[1] - p[1]) * (x[1] - p[1]));
    double z = x[2] - p[2];
    double R = p[3], H = p[4];
    // base segment (0,0)-(R,0)
    double bq = std::min(std::max(q, 0.0), R);
    double d2 = (q - bq) * (q - bq) + z * z;
    // slant segment (R,0)-(0,H)
    double ex = -R, ez = H;
    double t = ((q - R) * ex + z * ez) / (ex * ex + ez * ez);
    t = std::min(std::max(t, 0.0), 1.0);
    double sx = q - (R + t * ex), sz = z - t * ez;
    d2 = std::min(d2, sx * sx + sz * sz);
    bool inside = z >= 0.0 && z <= H && q <= R * (1.0 - z / H);
    double d = std::sqrt(d2);
    return inside ? -d : d;
}

// Distance from x to the solid, positive in the fluid.  The map's distance
// grid stores its negative (fluid side negative, as SetBox stores the box's
// signed distance), so that distWall = -tex3D(...) > 0 in the fluid.
float solid_distance(const OrcBoundaryDesc& D, const float* xf) {
    double x[3] = {xf[0], xf[1], xf[2]};
    double s = 1e30;
    for (int i = 0; i < D.numShapes; i++) {
        const OrcShape& S = D.shapes[i];
        double d;
        if (S.kind == 1) {
            double dx = x[0] - S.p[0], dy = x[1] - S.p[1], dz = x[2] - S.p[2];
            d = std::sqrt(dx * dx + dy * dy + dz * dz) - S.p[3];
        } else if (S.kind == 2) {
            d = cone_sdf(x, S.p);
        } else {
            d = -(double)box_signed_distance(xf, S.p, S.p + 3);
        }
        s = std::min(s, d);
    }
    return (float)s;
}

const OrcShape* only_box(const OrcBoundaryDesc& D) {
    for (int i = 0; i < D.numShapes; i++)
        if (D.shapes[i].kind == 3) return &D.shapes[i];
    return nullptr;
}

// evaluateDensityKernel / evaluateViscosityKernel (SphInComplexShapes.cpp:666-690):
// the coefficients are formed in double (M_PI is a double) and rounded to float.
float eval_density_kernel(float sqDist, float h) {
    float coeff = (float)(315.0f / (64.0f * 3.14159265358979323846 * h * h * h * h * h * h * h * h * h));
    float sqh = h * h;
    float diff = sqh - sqDist;
    if (diff < 0.0f) return 0.0f;
    return coeff * diff * diff * diff;
}

float eval_viscosity_kernel(float sqDist, float h) {
    float dist = std::sqrt(sqDist);
    if (dist > h) return 0.0f;
    return (float)(45.0f / (3.14159265358979323846 * h * h * h * h * h * h) * (h - dist));
}

}  // namespace

extern "C" {

void orc_boundary_dims(const OrcBoundaryDesc* D, unsigned int* dims) {
    for (int a = 0; a < 3; a++)
        dims[a] = (unsigned int)((D->gridEnd[a] - D->gridStart[a]) / D->gridSpacing) + 1;
}

// SetBox (SphInComplexShapes.cpp:203-313) generalised to the solids above,
// followed by Create{Distance,Density,Viscosity}TextureData (:366-427).
// Kept nodes are those with |distance| < compactSupport (clamped to
// +-restDistance); every other node reads entry 0 (distance -restDistance,
// density 0, viscosity 0; reset(), :641-652).  Ghost particles sit on a lattice
// of pitch particleSpacing: for a box container it is SetBox's lattice over
// the box grown by compactSupport + particleSpacing (:232-260); otherwise it
// covers the map grid grown by the same margin.  A lattice point is a ghost
// when it is not strictly inside the fluid.  Each ghost splats poly6 (density)
// and the viscosity kernel onto kept nodes within its support (:269-304).
int orc_boundary_maps(const OrcBoundaryDesc* Dp, float* dist, float* dens, float* visc) {
    const OrcBoundaryDesc& D = *Dp;
    unsigned int dims[3];
    orc_boundary_dims(Dp, dims);
    size_t numNodes = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<unsigned int> indexGrid(numNodes, 0u);
    std::vector<float> dists(1, -D.restDistance), denss(1, 0.0f), viscs(1, 0.0f);
    auto nodePos = [&](long i, long j, long k, float* p) {
        p[0] = D.gridStart[0] + D.gridSpacing * (float)i;
        p[1] = D.gridStart[1] + D.gridSpacing * (float)j;
        p[2] = D.gridStart[2] + D.gridSpacing * (float)k;
    };
    auto index = [&](long i, long j, long k) -> size_t {
        return (size_t)i + dims[0] * ((size_t)j + (size_t)dims[1] * (size_t)k);
    };
    for (unsigned int i = 0; i < dims[0]; i++)
        for (unsigned int j = 0; j < dims[1]; j++)
            for (unsigned int k = 0; k < dims[2]; k++) {
                float pos[3];
                nodePos(i, j, k, pos);
                float d = -solid_distance(D, pos);
                if (std::fabs(d) < D.compactSupport) {
                    if (std::fabs(d) > D.restDistance) d = d / std::fabs(d) * D.restDistance;
                    dists.push_back(d);
                    indexGrid[index(i, j, k)] = (unsigned int)(dists.size() - 1);
                }
            }
    // ghost lattice
    float ps = D.particleSpacing;
    float margin = D.compactSupport + ps;
    float s[3];
    unsigned int cnt[3];
    const OrcShape* box = only_box(D);
    for (int a = 0; a < 3; a++) {
        if (box) {
            float ext = box->p[3 + a] + margin;
            s[a] = box->p[a] - ext;
            cnt[a] = (unsigned int)(2 * ext / ps);
        } else {
            float lo = D.gridStart[a] - margin;
            float len = (float)(dims[a] - 1) * D.gridSpacing + 2 * margin;
            s[a] = lo;
            cnt[a] = (unsigned int)(len / ps);
        }
    }
    denss.resize(dists.size(), 0.0f);
    viscs.resize(dists.size(), 0.0f);
    float h = D.compactSupport;
    for (unsigned int k = 0; k <= cnt[2]; k++)
        for (unsigned int j = 0; j <= cnt[1]; j++)
            for (unsigned int i = 0; i <= cnt[0]; i++) {
                float g[3] = {s[0] + (float)i * ps, s[1] + (float)j * ps, s[2] + (float)k * ps};
                bool ghost;
                if (box && D.numShapes == 1)
                    ghost = !inside_box(g, box->p, box->p + 3);
                else
                    ghost = solid_distance(D, g) <= 0.0f;
                if (!ghost) continue;
                long cs[3], ce[3];
                for (int a = 0; a < 3; a++) {
                    long lo = (long)(int)((g[a] - h - D.gridStart[a]) / D.gridSpacing);
                    long hi = (long)(int)((g[a] + h - D.gridStart[a]) / D.gridSpacing);
                    cs[a] = std::min(std::max(lo, 0L), (long)dims[a] - 1);
                    ce[a] = std::min(std::max(hi, 0L), (long)dims[a] - 1);
                }
                for (long kk = cs[2]; kk <= ce[2]; kk++)
                    for (long jj = cs[1]; jj <= ce[1]; jj++)
                        for (long ii = cs[0]; ii <= ce[0]; ii++) {
                            unsigned int node = indexGrid[index(ii, jj, kk)];
                            if (node == 0) continue;
                            float np[3];
                            nodePos(ii, jj, kk, np);
                            float dx = g[0] - np[0], dy = g[1] - np[1], dz = g[2] - np[2];
                            float sq = dx * dx + dy * dy + dz * dz;
                            denss[node] += eval_density_kernel(sq, h);
                            viscs[node] += eval_viscosity_kernel(sq, h);
                        }
            }
    float viscScale = D.viscosity * D.particleMass / D.restDensity;
    for (size_t i = 1; i < dists.size(); i++) {
        denss[i] *= D.particleMass;
        viscs[i] *= viscScale;
    }
    for (size_t n = 0; n < numNodes; n++) {
        unsigned int node = indexGrid[n];
        if (dist) dist[n] = dists[node];
        if (dens) dens[n] = denss[node];
        if (visc) visc[n] = viscs[node];
    }
    return 0;
}

}  // extern "C"

// =============================================================================
//  Two-scale pass (AdvanceTwoScale, particle_simulation.cu:2145-2182, and
//  AdvanceSubParticles, :2119-2143)
// =============================================================================
namespace {

// split region test (find_split_particles, :932-952; reference region
// 0.2 <= x <= 0.5 is the default AABB of the options)
template <class R>
bool in_split_region(const OrcOptions& O, const R* x) {
    for (int a = 0; a < 3; a++)
        if (!(x[a] >= R(O.splitMin[a]) && x[a] <= R(O.splitMax[a]))) return false;
    return true;
}

// initialize_sub_particles radius (:1057-1059): the radicand is formed in
// double (M_PI is a double) and stored as float; pow(r, 1.0f/3.0f) is
// evaluated in double and rounded once to float, identically on every
// platform.  Children are always placed in the reference's float arithmetic
// (also by the FP64 restatement), so both restatements refine the same
// children.
inline float child_radius(float mass, float density) {
    double rad = (double)(3.0f * mass) / (4.0 * 3.14159265358979323846 * (double)density);
    float radicand = (float)rad;
    return (float)std::pow((double)radicand, (double)(1.0f / 3.0f));
}

const float kDir[8][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1},
                          {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
const float kSqrt3Inv = (float)0.577350269;  // SQRT3INV, :1028

template <class R>
struct TwoScale {
    int n = 0;
    std::vector<unsigned char> state;
    std::vector<R> subPos, subVel, subAcc, subRho, subPrs;  // 8n slots
    std::vector<int> splitIds, boundaryIds, defaultIds, subIds;
    std::vector<int> subHash, sortedSubIds, subStart, subEnd;
    std::vector<R> subScaleAcc;  // rounding-error scale of the children's accelerations
    int subCells = 0;
    explicit TwoScale(int n_) : n(n_), state(n_, 0), subPos(24 * (size_t)n_, R(0)),
        subVel(24 * (size_t)n_, R(0)), subAcc(24 * (size_t)n_, R(0)), subRho(8 * (size_t)n_, R(0)),
        subPrs(8 * (size_t)n_, R(0)), subScaleAcc(8 * (size_t)n_, R(0)) {}
};

// computeParticleState (:2495-2504) with find_boundary_particles read as the
// race-free scatter: every particle that is split after find_split_particles
// marks all particles of its stencil within compactSupport (self included),
// with r^2 = rx*rx + ry*ry + rz*rz as the reference forms it (:1002-1007).
// (In the reference a split particle that a neighbour has already marked
// reads state 3 and does not propagate -- an order-dependent outcome.)
template <class R>
void particle_state(const OrcParams& P, const OrcOptions& O, TwoScale<R>& T, const R* pos, const int* ids,
                    const int* start, const int* end) {
    const int n = T.n;
    for (int i = 0; i < n; i++) T.state[i] = (unsigned char)(T.state[i] << 2);
    for (int u = 0; u < n; u++) {
        int id = ids[u];
        if (in_split_region<R>(O, pos + 3 * (size_t)id)) T.state[id] |= 1;
    }
    std::vector<unsigned char> split(n);
    for (int i = 0; i < n; i++) split[i] = (T.state[i] & 3) == 1;
    Level<R> L = coarse_level<R>(P);
    R h2 = L.h * L.h;
    for (int u = 0; u < n; u++) {
        int id = ids[u];
        if (!split[id]) continue;
        const R* xs = pos + 3 * (size_t)id;
        for_each_cell<R>(P, xs, L.h, L.spacing, L.dim, start, end, [&](int s, int e) {
            for (int t = s; t < e; t++) {
                int v = ids[t];
                const R* xv = pos + 3 * (size_t)v;
                R rx = xs[0] - xv[0], ry = xs[1] - xv[1], rz = xs[2] - xv[2];
                R rn = rx * rx + ry * ry + rz * rz;
                if (rn <= h2) T.state[v] |= 2;
            }
        });
    }
}

// collect (:2509-2567) + collect_ids (:1118-1162): stable three-way split.
template <class R>
void collect(TwoScale<R>& T) {
    T.splitIds.clear();
    T.boundaryIds.clear();
    T.defaultIds.clear();
    for (int i = 0; i < T.n; i++) {
        int c = T.state[i] & 3;
        if (c == 0) T.defaultIds.push_back(i);
        else if (c == 2) T.boundaryIds.push_back(i);
        else T.splitIds.push_back(i);
    }
    T.subIds.clear();
    for (int p : T.splitIds)
        for (int k = 0; k < 8; k++) T.subIds.push_back(8 * p + k);
    for (int p : T.boundaryIds)
        for (int k = 0; k < 8; k++) T.subIds.push_back(8 * p + k);
}

// Class of a 2-bit state: 1 split (bit 0, collect's c == 1 || c == 3),
// 2 boundary, 0 default.
inline int state_class(int c) { return (c & 1) ? 1 : (c == 2 ? 2 : 0); }

// Merge-back (childMode 1; no reference counterpart): a parent whose class
// changes from split to boundary or default takes the mean position and
// velocity of its eight children (summed in slot order, times 1/8) before its
// coarse integration.  Its coarse acceleration stays the one computed at its
// own position.
template <class R>
void merge_back(TwoScale<R>& T, R* pos, R* vel) {
    for (int i = 0; i < T.n; i++) {
        int code = T.state[i] & 15;
        if (state_class(code >> 2) != 1 || state_class(code & 3) == 1) continue;
        for (int a = 0; a < 3; a++) {
            R sx = R(0), sv = R(0);
            for (int k = 0; k < 8; k++) {
                sx += T.subPos[3 * (8 * (size_t)i + k) + a];
                sv += T.subVel[3 * (8 * (size_t)i + k) + a];
            }
            pos[3 * (size_t)i + a] = sx * R(0.125);
            vel[3 * (size_t)i + a] = sv * R(0.125);
        }
    }
}

// initialize_sub_particles (:1023-1090) for split and boundary parents; with
// childMode 1 only for parents whose class changed (the transitions that
// the reference lists at :1052-1055 and leaves commented out).
template <class R>
void init_children(const OrcParams& P, const OrcOptions& O, TwoScale<R>& T, const R* pos, const R* vel,
                   const R* rho) {
    auto seed = [&](int id) {
        float radius = child_radius(P.particleMass, (float)rho[id]);
        for (int k = 0; k < 8; k++) {
            size_t slot = 8 * (size_t)id + k;
            for (int a = 0; a < 3; a++) {
                T.subVel[3 * slot + a] = vel[3 * (size_t)id + a];
                // pos + dir*radius, contracted to one fused multiply-add as
                // nvcc contracts it in the reference's kernel (:1080-1085)
                float d = kDir[k][a] * kSqrt3Inv;
                T.subPos[3 * slot + a] = R(std::fmaf(d, radius, (float)pos[3 * (size_t)id + a]));
            }
        }
    };
    auto changed = [&](int id) {
        int code = T.state[id] & 15;
        return O.childMode == 0 || state_class(code >> 2) != state_class(code & 3);
    };
    for (int p : T.splitIds)
        if (changed(p)) seed(p);
    for (int p : T.boundaryIds)
        if (changed(p)) seed(p);
}

// project_quantities (:570-622, 1328-1381): unweighted mean of the coarse
// density and pressure within compactSupportSub, searched on the coarse grid.
// A child with no coarse particle in reach gets 0 (the reference divides 0 by 0).
template <class R>
void project(const OrcParams& P, TwoScale<R>& T, const R* pos, const R* rho, const R* prs, const int* ids,
             const int* start, const int* end) {
    const int nSplit = (int)T.splitIds.size();
    R hs = R(P.compactSupportSub);
    R hs2 = hs * hs;
    R spacing = R(P.gridSpacing);
    for (size_t idx = 8 * (size_t)nSplit; idx < T.subIds.size(); idx++) {
        size_t slot = (size_t)T.subIds[idx];
        const R* x = &T.subPos[3 * slot];
        R d = R(0), p = R(0), count = R(0);
        for_each_cell<R>(P, x, hs, spacing, P.gridDim, start, end, [&](int s, int e) {
            for (int t = s; t < e; t++) {
                int j = ids[t];
                const R* xj = pos + 3 * (size_t)j;
                R dx = x[0] - xj[0], dy = x[1] - xj[1], dz = x[2] - xj[2];
                R sq = dx * dx + dy * dy + dz * dz;
                if (sq <= hs2) {
                    d += rho[j];
                    p += prs[j];
                    count += R(1);
                }
            }
        });
        T.subRho[slot] = count > R(0) ? d / count : R(0);
        T.subPrs[slot] = count > R(0) ? p / count : R(0);
    }
}

// The fine level (:2327-2437, 2464-2493): hash, sort, cells, density and
// forces of the regular children, integration and collision of all children.
template <class R>
void sub_level_step(const OrcParams& P, const OrcOptions& O, TwoScale<R>& T, bool density, bool forces) {
    Level<R> L = sub_level<R>(P);
    const int nSub = (int)T.subIds.size();
    const int nReg = 8 * (int)T.splitIds.size();
    T.subCells = num_cells(P.gridDimSubParticles);
    T.subHash.assign(nSub, 0);
    T.sortedSubIds = T.subIds;
    for (int idx = 0; idx < nSub; idx++)
        particle_hash<R>(&T.subPos[3 * (size_t)T.subIds[idx]], P.gridOrigin, L.spacing, L.dim, &T.subHash[idx]);
    std::vector<int> sh = T.subHash;
    stable_sort_by_hash(sh.data(), T.sortedSubIds.data(), nSub, T.subCells);
    T.subStart.assign(T.subCells, EMPTY);
    T.subEnd.assign(T.subCells, EMPTY);
    if (nSub > 0) cell_start_end(sh.data(), nSub, T.subCells, T.subStart.data(), T.subEnd.data());
    T.subHash = sh;
    if (density) {
        for (int idx = 0; idx < nReg; idx++) {
            size_t slot = (size_t)T.subIds[idx];
            density_one<R>(P, L, nullptr, false, T.subPos.data(), T.sortedSubIds.data(), T.subStart.data(),
                           T.subEnd.data(), &T.subPos[3 * slot], &T.subRho[slot], &T.subPrs[slot]);
        }
    }
    if (forces) {
        for (int idx = 0; idx < nReg; idx++) {
            size_t slot = (size_t)T.subIds[idx];
            force_one<R>(P, O, L, nullptr, true, T.subPos.data(), T.subVel.data(), T.subRho.data(),
                         T.subPrs.data(), T.sortedSubIds.data(), T.subStart.data(), T.subEnd.data(), slot,
                         &T.subAcc[3 * slot], &T.subScaleAcc[slot]);
        }
    }
}

template <class R>
void sub_integrate_collide(const OrcParams& P, TwoScale<R>& T) {
    R dt = R(P.timeStepSubParticles);
    for (int slot : T.subIds) {
        integrate_one<R>(dt, &T.subAcc[3 * (size_t)slot], &T.subPos[3 * (size_t)slot], &T.subVel[3 * (size_t)slot]);
        collide_one<R>(P, &T.subPos[3 * (size_t)slot], &T.subVel[3 * (size_t)slot]);
    }
}

template <class R>
int step_two_scale(const OrcParams& P, const OrcOptions& O, const OrcMaps* M, TwoScale<R>& T, R* pos, R* vel,
                   R* rho, R* prs, R* acc, int* hash, int* ids, int* start, int* end) {
    const int n = T.n;
    Level<R> L = coarse_level<R>(P);
    int C = num_cells(P.gridDim);
    if (hash_all<R>(P, L, pos, n, hash, ids)) return 1;
    if (!stable_sort_by_hash(hash, ids, n, C)) return 2;
    cell_start_end(hash, n, C, start, end);
    for (int i = 0; i < n; i++)
        density_one<R>(P, L, M, true, pos, ids, start, end, pos + 3 * (size_t)i, &rho[i], &prs[i]);
    for (int i = 0; i < n; i++)
        force_one<R>(P, O, L, M, false, pos, vel, rho, prs, ids, start, end, (size_t)i, acc + 3 * (size_t)i,
                     nullptr);
    particle_state<R>(P, O, T, pos, ids, start, end);
    if (O.childMode == 1) merge_back<R>(T, pos, vel);
    collect<R>(T);
    init_children<R>(P, O, T, pos, vel, rho);
    project<R>(P, T, pos, rho, prs, ids, start, end);
    sub_level_step<R>(P, O, T, true, true);
    for (int i = 0; i < n; i++)
        integrate_one<R>(R(P.timeStep), acc + 3 * (size_t)i, pos + 3 * (size_t)i, vel + 3 * (size_t)i);
    // integrateSubParticles + handleSubParticleCollisions act on each child
    // alone, so they are fused per child; the coarse collision likewise
    sub_integrate_collide<R>(P, T);
    for (int i = 0; i < n; i++) collide_one<R>(P, pos + 3 * (size_t)i, vel + 3 * (size_t)i);
    return 0;
}

// The two-scale part of AdvanceTwoScale (:2157-2171) from given coarse
// results: pre-integration positions and velocities, densities and
// pressures, and the coarse sort and cell tables.
template <class R>
int two_scale_part(const OrcParams& P, const OrcOptions& O, TwoScale<R>& T, const R* pos, const R* vel,
                   const R* rho, const R* prs, const int* ids, const int* start, const int* end) {
    particle_state<R>(P, O, T, pos, ids, start, end);
    std::vector<R> mpos(pos, pos + 3 * (size_t)T.n), mvel(vel, vel + 3 * (size_t)T.n);
    if (O.childMode == 1) merge_back<R>(T, mpos.data(), mvel.data());
    collect<R>(T);
    init_children<R>(P, O, T, mpos.data(), mvel.data(), rho);
    project<R>(P, T, mpos.data(), rho, prs, ids, start, end);
    sub_level_step<R>(P, O, T, true, true);
    sub_integrate_collide<R>(P, T);
    return 0;
}

// AdvanceSubParticles (:2119-2143) on the current lists: fine hash, sort,
// cells, density, projection, forces, integration and collision.
template <class R>
int step_sub_only(const OrcParams& P, const OrcOptions& O, TwoScale<R>& T, const R* pos, const R* rho,
                  const R* prs, const int* ids, const int* start, const int* end) {
    sub_level_step<R>(P, O, T, true, false);
    project<R>(P, T, pos, rho, prs, ids, start, end);
    sub_level_step<R>(P, O, T, false, true);
    sub_integrate_collide<R>(P, T);
    return 0;
}

}  // namespace

// =============================================================================
//  C entry points of the two-scale pass
// =============================================================================
extern "C" {

struct OrcTwoScale;  // opaque: TwoScale<float> or TwoScale<double>

void* orc_ts_new(int n, int fp64) {
    if (fp64) return new TwoScale<double>(n);
    return new TwoScale<float>(n);
}

void orc_ts_free(void* h, int fp64) {
    if (fp64) delete static_cast<TwoScale<double>*>(h);
    else delete static_cast<TwoScale<float>*>(h);
}

// mode 1: AdvanceTwoScale; coarse state updated in place, coarse outputs filled.
int orc_ts_step_f32(void* h, const OrcParams* P, const OrcOptions* O, const OrcMaps* M, float* pos, float* vel,
                    float* rho, float* prs, float* acc, int* hash, int* ids, int* start, int* end) {
    return step_two_scale<float>(*P, *O, M, *static_cast<TwoScale<float>*>(h), pos, vel, rho, prs, acc, hash, ids,
                                 start, end);
}

int orc_ts_step_f64(void* h, const OrcParams* P, const OrcOptions* O, const OrcMaps* M, double* pos, double* vel,
                    double* rho, double* prs, double* acc, int* hash, int* ids, int* start, int* end) {
    return step_two_scale<double>(*P, *O, M, *static_cast<TwoScale<double>*>(h), pos, vel, rho, prs, acc, hash,
                                  ids, start, end);
}

int orc_ts_sub_only_f32(void* h, const OrcParams* P, const OrcOptions* O, const float* pos, const float* rho,
                        const float* prs, const int* ids, const int* start, const int* end) {
    return step_sub_only<float>(*P, *O, *static_cast<TwoScale<float>*>(h), pos, rho, prs, ids, start, end);
}

int orc_ts_sub_only_f64(void* h, const OrcParams* P, const OrcOptions* O, const double* pos, const double* rho,
                        const double* prs, const int* ids, const int* start, const int* end) {
    return step_sub_only<double>(*P, *O, *static_cast<TwoScale<double>*>(h), pos, rho, prs, ids, start, end);
}

int orc_ts_part_f32(void* h, const OrcParams* P, const OrcOptions* O, const float* pos, const float* vel,
                    const float* rho, const float* prs, const int* ids, const int* start, const int* end) {
    return two_scale_part<float>(*P, *O, *static_cast<TwoScale<float>*>(h), pos, vel, rho, prs, ids, start, end);
}

int orc_ts_part_f64(void* h, const OrcParams* P, const OrcOptions* O, const double* pos, const double* vel,
                    const double* rho, const double* prs, const int* ids, const int* start, const int* end) {
    return two_scale_part<double>(*P, *O, *static_cast<TwoScale<double>*>(h), pos, vel, rho, prs, ids, start,
                                  end);
}

// counts: split, boundary, default, sub-particles, sub cells
void orc_ts_counts(void* h, int fp64, int* out) {
    auto fill = [&](auto& T) {
        out[0] = (int)T.splitIds.size();
        out[1] = (int)T.boundaryIds.size();
        out[2] = (int)T.defaultIds.size();
        out[3] = (int)T.subIds.size();
        out[4] = T.subCells;
    };
    if (fp64) fill(*static_cast<TwoScale<double>*>(h));
    else fill(*static_cast<TwoScale<float>*>(h));
}

// what: 0 state (uint8[n]), 1 split ids, 2 boundary ids, 3 default ids,
// 4 sub ids, 5 sub hash (sorted), 6 sorted sub ids, 7 sub cell start,
// 8 sub cell end (int arrays); 10 sub positions, 11 sub velocities,
// 12 sub accelerations (R[8n*3]), 13 sub density, 14 sub pressure (R[8n]);
// 20 state (write, uint8[n]).
void orc_ts_get(void* h, int fp64, int what, void* dst) {
    auto get = [&](auto& T) {
        using R = typename std::remove_reference<decltype(T.subPos[0])>::type;
        auto ci = [&](const std::vector<int>& v) { std::memcpy(dst, v.data(), sizeof(int) * v.size()); };
        auto cr = [&](const std::vector<R>& v) { std::memcpy(dst, v.data(), sizeof(R) * v.size()); };
        switch (what) {
            case 0: std::memcpy(dst, T.state.data(), T.state.size()); break;
            case 1: ci(T.splitIds); break;
            case 2: ci(T.boundaryIds); break;
            case 3: ci(T.defaultIds); break;
            case 4: ci(T.subIds); break;
            case 5: ci(T.subHash); break;
            case 6: ci(T.sortedSubIds); break;
            case 7: ci(T.subStart); break;
            case 8: ci(T.subEnd); break;
            case 10: cr(T.subPos); break;
            case 11: cr(T.subVel); break;
            case 12: cr(T.subAcc); break;
            case 13: cr(T.subRho); break;
            case 14: cr(T.subPrs); break;
            case 15: cr(T.subScaleAcc); break;
            case 20: std::memcpy(T.state.data(), dst, T.state.size()); break;
            case 21: std::memcpy(T.subPos.data(), dst, sizeof(R) * T.subPos.size()); break;
            case 22: std::memcpy(T.subVel.data(), dst, sizeof(R) * T.subVel.size()); break;
        }
    };
    if (fp64) get(*static_cast<TwoScale<double>*>(h));
    else get(*static_cast<TwoScale<float>*>(h));
}

}  // extern "C"

// =============================================================================
//  Mesh signed distance grid (BoundaryMap::computeSignedDistanceField,
//  boundary_map.cpp:351-470; PointInMeshTest::isContained,
//  point_in_mesh_test.cpp:31-120), brute force in double precision.  The
//  closest point is found here by projecting onto the triangle's plane when
//  the projection falls inside the triangle, else on the nearest of the three
//  edges; the sign is the parity of the crossings of the ray o + t (0.3137 dx,
//  0.2718 dx, max(mesh height, dx)), t > 0, with every triangle, solved by
//  Cramer's rule.  Nodes outside the mesh's bounding box are outside.
// =============================================================================
namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

V3 closest_on_segment(V3 p, V3 a, V3 b) {
    V3 ab = b - a;
    double l2 = dot(ab, ab);
    double t = l2 > 0.0 ? dot(p - a, ab) / l2 : 0.0;
    t = std::min(1.0, std::max(0.0, t));
    return a + t * ab;
}

V3 closest_on_triangle_oracle(V3 p, V3 a, V3 b, V3 c) {
    V3 nrm = cross(b - a, c - a);
    double n2 = dot(nrm, nrm);
    if (n2 > 0.0) {
        V3 q = p - (dot(p - a, nrm) / n2) * nrm;  // projection onto the plane
        // inside test by the signs of the sub-triangle normals
        double s0 = dot(cross(b - a, q - a), nrm), s1 = dot(cross(c - b, q - b), nrm),
               s2 = dot(cross(a - c, q - c), nrm);
        if (s0 >= 0.0 && s1 >= 0.0 && s2 >= 0.0) return q;
    }
    V3 best = closest_on_segment(p, a, b);
    for (V3 cand : {closest_on_segment(p, b, c), closest_on_segment(p, c, a)})
        if (dot(p - cand, p - cand) < dot(p - best, p - best)) best = cand;
    return best;
}

bool ray_hits_oracle(V3 o, V3 d, V3 a, V3 b, V3 c) {
    // o + t d = a + u (b - a) + v (c - a): 3x3 system in (t, u, v)
    V3 e1 = b - a, e2 = c - a, r = o - a;
    V3 m0 = {-d.x, -d.y, -d.z};
    double det = dot(m0, cross(e1, e2));
    if (det == 0.0) return false;
    double t = dot(r, cross(e1, e2)) / det;
    double u = dot(m0, cross(r, e2)) / det;
    double v = dot(m0, cross(e1, r)) / det;
    return t > 0.0 && u >= 0.0 && v >= 0.0 && u + v <= 1.0;
}

}  // namespace

extern "C" void orc_mesh_sdf(const float* verts, int nv, const unsigned int* faces, int nf, const float* origin,
                             float dx, const unsigned int* dims, float maxDist, float* dist, float* normal) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < nv; i++)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], (double)verts[3 * i + a]);
            hi[a] = std::max(hi[a], (double)verts[3 * i + a]);
        }
    const V3 ray = {0.3137 * dx, 0.2718 * dx, std::max(hi[2] - lo[2], (double)dx)};
    auto vert = [&](unsigned int k) { return V3{verts[3 * k], verts[3 * k + 1], verts[3 * k + 2]}; };
    const size_t n = (size_t)dims[0] * dims[1] * dims[2];
    for (size_t id = 0; id < n; id++) {
        const unsigned int i = (unsigned int)(id % dims[0]), j = (unsigned int)((id / dims[0]) % dims[1]),
                           k = (unsigned int)(id / ((size_t)dims[0] * dims[1]));
        const float xf[3] = {origin[0] + (float)i * dx, origin[1] + (float)j * dx, origin[2] + (float)k * dx};
        const V3 x = {xf[0], xf[1], xf[2]};
        double best = 1e300;
        V3 q = {0, 0, 0};
        for (int f = 0; f < nf; f++) {
            V3 c = closest_on_triangle_oracle(x, vert(faces[3 * f]), vert(faces[3 * f + 1]), vert(faces[3 * f + 2]));
            double d = std::sqrt(dot(x - c, x - c));
            if (d < best) {
                best = d;
                q = c;
            }
        }
        const bool band = best <= (double)maxDist;
        bool inside = false;
        if (x.x >= lo[0] && x.x <= hi[0] && x.y >= lo[1] && x.y <= hi[1] && x.z >= lo[2] && x.z <= hi[2]) {
            unsigned int cnt = 0;
            for (int f = 0; f < nf; f++)
                cnt += ray_hits_oracle(x, ray, vert(faces[3 * f]), vert(faces[3 * f + 1]), vert(faces[3 * f + 2]));
            inside = cnt & 1u;
        }
        const double mag = band ? best : (double)maxDist;
        dist[id] = (float)(inside ? -mag : mag);
        if (normal) {
            for (int a = 0; a < 3; a++) normal[3 * id + a] = 0.0f;
            if (band && best > 0.0) {
                V3 r = (1.0 / best) * (x - q);
                normal[3 * id] = (float)r.x;
                normal[3 * id + 1] = (float)r.y;
                normal[3 * id + 2] = (float)r.z;
            }
        }
    }
}
