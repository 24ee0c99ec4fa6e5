// Per-particle input features of the learned step corrector, aggregated over
// the neighbours within h of the sorted pre-step state (the copies the force
// stage reads and leaves untouched).  24 FP32 values per particle:
//
//   0      rho/rho0 - 1
//   1      Shepard sum  sum_j (m/rho_j) W_ij           (poly6, j != i)
//   2-4    v                                            (m/s)
//   5-7    a / g                                        (this step's acceleration)
//   8-10   sum_j (m/rho_j) W_ij (v_j - v_i)            (m/s)
//   11     dtL * sum_j (m/rho_j) (v_j - v_i) . gradW_ij (spiky gradient)
//   12-14  dtL * sum_j (m/rho_j) (v_j - v_i) x gradW_ij
//   15-17  h * sum_j (m/rho_j) gradW_ij                 (colour-field gradient)
//   18     neighbour count / 32
//   19     wall distance / h, capped at 4               (box walls, boundary map)
//   20-22  unit wall normal, pointing into the fluid
//   23     |v| dtL / h                                  (Courant number)
//
// dtL is the learned step (stride * dt).  No reference counterpart.
#include "sph_corrector.h"
#include "sph_device.cuh"

namespace sph {

namespace {

__global__ void __launch_bounds__(128) k_features(int n, const float4* __restrict__ posS,
                                                  const float4* __restrict__ velS,
                                                  const float4* __restrict__ rho4S,
                                                  const float4* __restrict__ accS,
                                                  const int* __restrict__ workIds, RowTables T, GridDev g,
                                                  PhysDev ph, MapDev map, int boxWalls, float dtL, int byId,
                                                  float* __restrict__ feat) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    const float4 xi = posS[u], vi = velS[u], ri = rho4S[u], ai = accS[u];
    const float h = ph.h, h2 = ph.h2;
    const float gw = -ph.pressCoef;  // mass * gradSpiky
    const Stencil st = stencil(xi, h, g);
    float shep = 0.f, mx = 0.f, my = 0.f, mz = 0.f, div = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    float gx = 0.f, gy = 0.f, gz = 0.f, cnt = 0.f;
    for (int r = 0; r < 9; r++) {
        int s, e;
        row_range(xi, st, h, g, T, true, r, s, e);
        for (int j = s; j < e; j++) {
            if (j == u) continue;
            const float4 xj = posS[j];
            const float r2 = dist2(xi, xj);
            if (!(r2 < h2) || !(r2 > 0.f)) continue;
            const float4 rj = rho4S[j], vj = velS[j];
            const float inv = rj.w;  // 1/rho_j
            const float q = h2 - r2;
            const float w = ph.poly6m * q * q * q * inv;
            const float rr = sqrtf(r2);
            const float d = h - rr;
            const float gs = gw * d * d / rr * inv;
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float ux = vj.x - vi.x, uy = vj.y - vi.y, uz = vj.z - vi.z;
            const float ex = gs * dx, ey = gs * dy, ez = gs * dz;
            shep += w;
            mx += w * ux;
            my += w * uy;
            mz += w * uz;
            div += ux * ex + uy * ey + uz * ez;
            cx += uy * ez - uz * ey;
            cy += uz * ex - ux * ez;
            cz += ux * ey - uy * ex;
            gx += ex;
            gy += ey;
            gz += ez;
            cnt += 1.f;
        }
    }
    // nearest wall: the box container, and the boundary map where it is nearer
    float dw = 4.f * h, nx = 0.f, ny = 0.f, nz = 0.f;
    if (boxWalls) {
        const float c[3] = {xi.x - ph.boxCen[0], xi.y - ph.boxCen[1], xi.z - ph.boxCen[2]};
        for (int a = 0; a < 3; a++) {
            const float da = ph.boxDim[a] - fabsf(c[a]);
            if (da < dw) {
                dw = da;
                nx = a == 0 ? (c[a] > 0.f ? -1.f : 1.f) : 0.f;
                ny = a == 1 ? (c[a] > 0.f ? -1.f : 1.f) : 0.f;
                nz = a == 2 ? (c[a] > 0.f ? -1.f : 1.f) : 0.f;
            }
        }
    }
    if (map.present) {
        float uvw[3];
        map_uvw(map, xi, uvw);
        const float dm = -tri_scalar(map, map.dist, uvw[0], uvw[1], uvw[2]);
        if (dm < dw) {
            const float g0 = tri_scalar(map, map.dist, uvw[0] + map.du[0], uvw[1], uvw[2]) -
                             tri_scalar(map, map.dist, uvw[0] - map.du[0], uvw[1], uvw[2]);
            const float g1 = tri_scalar(map, map.dist, uvw[0], uvw[1] + map.du[1], uvw[2]) -
                             tri_scalar(map, map.dist, uvw[0], uvw[1] - map.du[1], uvw[2]);
            const float g2 = tri_scalar(map, map.dist, uvw[0], uvw[1], uvw[2] + map.du[2]) -
                             tri_scalar(map, map.dist, uvw[0], uvw[1], uvw[2] - map.du[2]);
            const float gn = sqrtf(g0 * g0 + g1 * g1 + g2 * g2);
            dw = dm;
            if (gn > 0.f) {
                nx = -g0 / gn;
                ny = -g1 / gn;
                nz = -g2 / gn;
            } else {
                nx = ny = nz = 0.f;
            }
        }
    }
    dw = fminf(fmaxf(dw, 0.f), 4.f * h);
    const float gInv = ph.gravity != 0.f ? 1.f / ph.gravity : 1.f;
    const float vn = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z);
    float4* dst = reinterpret_cast<float4*>(feat + (size_t)(byId ? workIds[u] : u) * mlp::IN);
    dst[0] = make_float4(ri.x / ph.restDensity - 1.f, shep, vi.x, vi.y);
    dst[1] = make_float4(vi.z, ai.x * gInv, ai.y * gInv, ai.z * gInv);
    dst[2] = make_float4(mx, my, mz, div * dtL);
    dst[3] = make_float4(cx * dtL, cy * dtL, cz * dtL, gx * h);
    dst[4] = make_float4(gy * h, gz * h, cnt * (1.f / 32.f), dw / h);
    dst[5] = make_float4(nx, ny, nz, vn * dtL / h);
}

}  // namespace

void launch_features(int n, const float4* posS, const float4* velS, const float4* rho4S, const float4* accS,
                     const int* workIds, RowTables T, GridDev g, PhysDev ph, MapDev map, int boxWalls,
                     float dtL, int byId, float* feat, cudaStream_t s) {
    if (n > 0)
        k_features<<<(n + 127) / 128, 128, 0, s>>>(n, posS, velS, rho4S, accS, workIds, T, g, ph, map, boxWalls,
                                                   dtL, byId, feat);
}

}  // namespace sph
