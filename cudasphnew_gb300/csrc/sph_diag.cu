// FP64 conservation diagnostics of the coarse level: mass, momentum, kinetic
// and potential energy of the current state, and the density statistics of
// the last density pass.  The reference has no counterpart; its simulation
// data reserves an "energy" column (particle_simulation.h:40-51) that it
// never fills.
//
// Deterministic: every block reduces a fixed particle range in a fixed tree
// order into one row of partials, and one block sums the rows in order, so
// the result depends only on n and the launch shape (fixed here).
#include "sph_internal.h"

namespace sph {

namespace {

constexpr int DIAG_THREADS = 256;
constexpr int DIAG_BLOCKS = 304;  // 2 per SM on 152 SMs

__device__ __forceinline__ void block_sum(double* sh, double v[DIAG_TERMS], bool maxLast) {
    const int t = threadIdx.x;
    for (int k = 0; k < DIAG_TERMS; k++) sh[k * DIAG_THREADS + t] = v[k];
    __syncthreads();
    for (int w = DIAG_THREADS / 2; w > 0; w >>= 1) {
        if (t < w)
            for (int k = 0; k < DIAG_TERMS; k++) {
                double a = sh[k * DIAG_THREADS + t], b = sh[k * DIAG_THREADS + t + w];
                sh[k * DIAG_THREADS + t] = (maxLast && k == DIAG_TERMS - 1) ? fmax(a, b) : a + b;
            }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(DIAG_THREADS) k_diag_partial(int n, const float4* __restrict__ pos,
                                                              const float4* __restrict__ vel,
                                                              const float4* __restrict__ rho4S, int haveRho,
                                                              double mass, double gravity, double rest0,
                                                              int axis, double* __restrict__ partial) {
    __shared__ double sh[DIAG_TERMS * DIAG_THREADS];
    double v[DIAG_TERMS];
    for (int k = 0; k < DIAG_TERMS; k++) v[k] = 0.0;
    // contiguous range per block, strided by thread inside it
    const long long per = ((long long)n + gridDim.x - 1) / gridDim.x;
    const long long lo = per * blockIdx.x;
    const long long hi = min((long long)n, lo + per);
    for (long long i = lo + threadIdx.x; i < hi; i += DIAG_THREADS) {
        float4 x = pos[i], u = vel[i];
        double ux = u.x, uy = u.y, uz = u.z;
        double xa = axis == 0 ? (double)x.x : axis == 1 ? (double)x.y : (double)x.z;
        v[DIAG_MASS] += mass;
        v[DIAG_MOM_X] += mass * ux;
        v[DIAG_MOM_Y] += mass * uy;
        v[DIAG_MOM_Z] += mass * uz;
        v[DIAG_KINETIC] += 0.5 * mass * (ux * ux + uy * uy + uz * uz);
        v[DIAG_POTENTIAL] += mass * gravity * xa;
        if (haveRho) {
            double r = rho4S[i].x;
            v[DIAG_RHO_SUM] += r;
            v[DIAG_RHO_MAXERR] = fmax(v[DIAG_RHO_MAXERR], fabs(r - rest0) / rest0);
        }
    }
    block_sum(sh, v, true);
    if (threadIdx.x == 0)
        for (int k = 0; k < DIAG_TERMS; k++) partial[(size_t)blockIdx.x * DIAG_TERMS + k] = sh[k * DIAG_THREADS];
}

__global__ void __launch_bounds__(DIAG_THREADS) k_diag_final(int blocks, const double* __restrict__ partial,
                                                            double* __restrict__ out) {
    __shared__ double sh[DIAG_TERMS * DIAG_THREADS];
    double v[DIAG_TERMS];
    for (int k = 0; k < DIAG_TERMS; k++) v[k] = 0.0;
    for (int b = threadIdx.x; b < blocks; b += DIAG_THREADS)
        for (int k = 0; k < DIAG_TERMS; k++) {
            double p = partial[(size_t)b * DIAG_TERMS + k];
            v[k] = k == DIAG_RHO_MAXERR ? fmax(v[k], p) : v[k] + p;
        }
    block_sum(sh, v, true);
    if (threadIdx.x == 0)
        for (int k = 0; k < DIAG_TERMS; k++) out[k] = sh[k * DIAG_THREADS];
}

}  // namespace

int diag_partial_rows() { return DIAG_BLOCKS; }

void launch_diagnostics(int n, const float4* pos, const float4* vel, const float4* rho4S, int haveRho,
                        double mass, double gravity, double rest0, int axis, double* partial, double* out,
                        cudaStream_t s) {
    k_diag_partial<<<DIAG_BLOCKS, DIAG_THREADS, 0, s>>>(n, pos, vel, rho4S, haveRho, mass, gravity, rest0, axis,
                                                        partial);
    k_diag_final<<<1, DIAG_THREADS, 0, s>>>(DIAG_BLOCKS, partial, out);
}

}  // namespace sph
