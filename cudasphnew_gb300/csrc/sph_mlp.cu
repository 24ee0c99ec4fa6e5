// The learned step corrector's MLP on tcgen05 tensor cores: inference
// (k_mlp_apply), the fused forward + backward pass of one optimiser step
// (k_mlp_grad), Adam (k_mlp_adam), and the small reductions around them.
//
// Network: 24 features -> 64 -> 64 -> 6, SiLU between layers.  Weights and
// activations are BF16, products accumulate in FP32 in tensor memory (TMEM).
// One CTA of 128 threads works on tiles of 128 samples: thread t owns sample
// row t, which is TMEM lane t of every M = 128 accumulator.  One elected thread
// issues the MMAs; tcgen05.commit arrives on an mbarrier that it polls with
// an iteration limit, after which the kernel latches STATUS_DEVICE_WAIT, waits
// once more (bounded) for its MMAs, frees its TMEM and returns.
//
// The training kernel keeps the three weight-gradient accumulators in TMEM
// across all tiles of its CTA (dW = dZ^T X as an M = 128 MMA whose A operand
// is the transposed gradient written to shared memory; rows beyond the layer
// width are ignored), so a CTA writes one gradient row per optimiser step and
// Adam sums the rows in a fixed order: training is deterministic.
#include <cmath>

#include "sph_corrector.h"
#include "sph_device.cuh"
#include "sph_mlp_tile.cuh"
#include "sph_tc.cuh"

namespace sph {

namespace {

using namespace mlp;
using namespace tc;

// Normalised features of one sample (zeros for padding rows).
__device__ __forceinline__ void load_features(const float* __restrict__ feat, long long row, bool valid,
                                              const float* norm, float (&f)[INP]) {
#pragma unroll
    for (int k = 0; k < INP; k++) f[k] = 0.f;
    if (!valid) return;
    const float4* src = reinterpret_cast<const float4*>(feat + row * IN);
#pragma unroll
    for (int c = 0; c < IN / 4; c++) {
        const float4 q = src[c];
        f[4 * c + 0] = q.x;
        f[4 * c + 1] = q.y;
        f[4 * c + 2] = q.z;
        f[4 * c + 3] = q.w;
    }
    standardise(f, norm);
}

// ---------------------------------------------------------------------------
// Inference
// ---------------------------------------------------------------------------
constexpr int A_W = 0;                  // W1, W2, W3 (IMG_FWD_BYTES)
constexpr int A_X = 16384;              // 128 x 32
constexpr int A_H1 = A_X + 8192;        // 128 x 64
constexpr int A_H2 = A_H1 + 16384;      // 128 x 64
constexpr int A_BIAS = A_H2 + 16384;    // NBIAS floats
constexpr int A_NORM = A_BIAS + 4 * NBIAS;
constexpr int A_BAR = A_NORM + 4 * NNORM;  // MMA barrier, TMEM slot, weight-copy barrier
constexpr int A_SMEM = A_BAR + 32;
// Three CTAs fit an SM's shared memory; their 128-column TMEM allocations
// (3 x 128 <= 512) always fit beside each other.
constexpr int A_CTAS_PER_SM = 3;
constexpr int A_TMEM_COLS = 128;  // D1 at 0, D2 at 64, D3 reuses D1's columns
static_assert(A_CTAS_PER_SM * A_TMEM_COLS <= 512, "inference TMEM");

__global__ void __launch_bounds__(TILE, 1)
    k_mlp_apply(int n, const float* __restrict__ feat, MlpDev m, int mode, const int* __restrict__ workIds,
                float4* __restrict__ pos, float4* __restrict__ vel, PhysDev ph, int collideFlag,
                float* __restrict__ out, unsigned int* status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ int sOk;
    const int t = threadIdx.x, warp = t >> 5;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + A_BAR);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + A_BAR + 8);
    uint64_t* wbar = reinterpret_cast<uint64_t*>(sm + A_BAR + 16);
    float* sBias = reinterpret_cast<float*>(sm + A_BIAS);
    float* sNorm = reinterpret_cast<float*>(sm + A_NORM);
    for (int i = t; i < NBIAS; i += TILE) sBias[i] = epilogue_bias(m.bias, i);
    for (int i = t; i < NNORM; i += TILE) sNorm[i] = m.norm[i];
    if (t == 0) {
        mbar_init(bar, 1);
        mbar_init(wbar, 1);
        sOk = 1;
        // the weight image: one TMA bulk copy
        mbar_arrive_expect_tx(wbar, IMG_FWD_BYTES);
        bulk_g2s(sm + A_W, m.image, IMG_FWD_BYTES, wbar);
        if (!mbar_wait(wbar, 0, WAIT_LIMIT)) {
            sOk = 0;
            atomicOr(status, STATUS_DEVICE_WAIT);
            mbar_wait(wbar, 0, WAIT_LIMIT);  // once more for the copy in flight
        }
    }
    if (warp == 0) tmem_alloc(slot, A_TMEM_COLS);
    cta_sync();
    const uint32_t tbase = *slot;
    const uint32_t sW = smem_u32(sm + A_W);
    uint32_t phase = 0;
    const int tiles = (n + TILE - 1) / TILE;
    for (int tile = blockIdx.x; sOk && tile < tiles; tile += gridDim.x) {
        const long long u = (long long)tile * TILE + t;
        const bool valid = u < n;
        const long long row = (mode == 0 && valid) ? (long long)workIds[u] : u;
        {
            float f[INP];
            load_features(feat, row, valid, sNorm, f);
#pragma unroll
            for (int c = 0; c < INP / 8; c++) store_row8(sm + A_X, t, 8 * c, INP, f + 8 * c);
        }
        cta_sync();
        if (t == 0) mma_chain(tbase + 0, smem_u32(sm + A_X), sW + IMG_W1, INP, HID, false);
        if (!commit_and_wait(bar, phase, &sOk, t)) break;
        hidden_layer_out(tmem_at(tbase, 32 * warp, 0), sBias, sm + A_H1, t);
        cta_sync();
        if (t == 0) mma_chain(tbase + 64, smem_u32(sm + A_H1), sW + IMG_W2, HID, HID, false);
        if (!commit_and_wait(bar, phase, &sOk, t)) break;
        hidden_layer_out(tmem_at(tbase, 32 * warp, 64), sBias + HID, sm + A_H2, t);
        cta_sync();
        if (t == 0) mma_chain(tbase + 0, smem_u32(sm + A_H2), sW + IMG_W3, HID, OUTP, false);
        if (!commit_and_wait(bar, phase, &sOk, t)) break;
        float y[16];
        tmem_ld16(tmem_at(tbase, 32 * warp, 0), y);
        if (valid) {
            float c[OUT];
            decode_correction(sNorm, sBias + 2 * HID, y, c);
            if (mode == 0) {
                const int id = (int)row;
                const float4 p = pos[id], w = vel[id];
                float3 x = make_float3(p.x + c[0], p.y + c[1], p.z + c[2]);
                float3 v = make_float3(w.x + c[3], w.y + c[4], w.z + c[5]);
                if (collideFlag) collide(ph, x, v);
                pos[id] = make_float4(x.x, x.y, x.z, p.w);
                vel[id] = make_float4(v.x, v.y, v.z, 0.f);
            } else {
#pragma unroll
                for (int o = 0; o < OUT; o++) out[u * OUT + o] = c[o];
            }
        }
    }
    cta_sync();
    if (!sOk) drain(bar, phase, t, status);
    cta_sync();
    if (warp == 0) tmem_dealloc(tbase, A_TMEM_COLS);
}

// ---------------------------------------------------------------------------
// Training: forward + backward of the tiles of one optimiser step
// ---------------------------------------------------------------------------
constexpr int G_IMG = 0;                 // the whole image (IMG_BYTES)
constexpr int G_X = IMG_BYTES;           // 128 x 32   features
constexpr int G_XT = G_X + 8192;         // 32 x 128   features, transposed
constexpr int G_H1 = G_XT + 8192;        // 128 x 64
constexpr int G_H1T = G_H1 + 16384;      // 64 x 128
constexpr int G_H2 = G_H1T + 16384;      // 128 x 64
constexpr int G_H2T = G_H2 + 16384;      // 64 x 128
constexpr int G_P = G_H2T + 16384;       // 128 x 128  dY^T, dZ2^T, dZ1^T in turn
constexpr int G_Q = G_P + 32768;         // 128 x 64   dY (K = 16), dZ2 (K = 64) in turn
constexpr int G_BIAS = G_Q + 16384;
constexpr int G_NORM = G_BIAS + 4 * NBIAS;
constexpr int G_DB = G_NORM + 4 * NNORM;  // [4 warps][NBIAS] bias-gradient sums
constexpr int G_LOSS = G_DB + 4 * 4 * NBIAS;
constexpr int G_BAR = G_LOSS + 16;  // MMA barrier, TMEM slot, weight-copy barrier
constexpr int G_SMEM = G_BAR + 32;
static_assert(G_SMEM <= 227 * 1024, "training shared memory");

// TMEM columns (512 allocated; one CTA per SM).
constexpr int C_D1 = 0, C_D2 = 64, C_D3 = 128, C_G2 = 160, C_G1 = 224, C_DW3 = 288, C_DW2 = 352, C_DW1 = 416;

// Writes activation row t both as row t of a K = 64 operand and as column t
// of the transposed 64 x 128 operand.
__device__ __forceinline__ void store_both(unsigned char* sm, int rowOff, int colOff, int t, int k0,
                                           const float* v) {
    store_row8(sm + rowOff, t, k0, HID, v);
    store_row8(sm + rowOff, t, k0 + 8, HID, v + 8);
#pragma unroll
    for (int i = 0; i < 16; i++) store_bf16(sm + colOff, core_off(k0 + i, t, TILE), v[i]);
}

__device__ __forceinline__ void bias_grad(float* dbRow, int lane, int base, const float* v, int cnt) {
    for (int i = 0; i < cnt; i++) {
        const float s = warp_sum(v[i]);
        if (lane == 0) dbRow[base + i] += s;
    }
}

__global__ void __launch_bounds__(TILE, 1)
    k_mlp_grad(int tilesPerCta, const int* __restrict__ tileList, const float* __restrict__ feat,
               const float* __restrict__ tgt, long long count, float invScale, MlpDev m,
               float* __restrict__ partial, unsigned int* status) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ int sOk;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + G_BAR);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + G_BAR + 8);
    uint64_t* wbar = reinterpret_cast<uint64_t*>(sm + G_BAR + 16);
    float* sBias = reinterpret_cast<float*>(sm + G_BIAS);
    float* sNorm = reinterpret_cast<float*>(sm + G_NORM);
    float* sDb = reinterpret_cast<float*>(sm + G_DB);
    float* sLoss = reinterpret_cast<float*>(sm + G_LOSS);
    for (int i = t; i < NBIAS; i += TILE) sBias[i] = m.bias[i];
    for (int i = t; i < NNORM; i += TILE) sNorm[i] = m.norm[i];
    for (int i = t; i < 4 * NBIAS; i += TILE) sDb[i] = 0.f;
    if (t < 4) sLoss[t] = 0.f;
    if (t == 0) {
        mbar_init(bar, 1);
        mbar_init(wbar, 1);
        sOk = 1;
        // the weight image (with the transposes the backward pass reads): one TMA bulk copy
        mbar_arrive_expect_tx(wbar, IMG_BYTES);
        bulk_g2s(sm + G_IMG, m.image, IMG_BYTES, wbar);
        if (!mbar_wait(wbar, 0, WAIT_LIMIT)) {
            sOk = 0;
            atomicOr(status, STATUS_DEVICE_WAIT);
            mbar_wait(wbar, 0, WAIT_LIMIT);  // once more for the copy in flight
        }
    }
    if (warp == 0) tmem_alloc(slot, 512);
    cta_sync();
    const uint32_t tb = *slot;
    const uint32_t sImg = smem_u32(sm + G_IMG);
    float* dbRow = sDb + warp * NBIAS;
    uint32_t phase = 0;
    bool ok = sOk != 0;
    for (int j = 0; j < tilesPerCta && ok; j++) {
        const int tile = tileList[(size_t)blockIdx.x * tilesPerCta + j];
        const long long row = (long long)tile * TILE + t;
        const bool valid = row < count;
        float tn[OUT];
        {
            float f[INP];
            load_features(feat, row, valid, sNorm, f);
#pragma unroll
            for (int c = 0; c < INP / 8; c++) store_row8(sm + G_X, t, 8 * c, INP, f + 8 * c);
#pragma unroll
            for (int k = 0; k < INP; k++) store_bf16(sm + G_XT, core_off(k, t, TILE), f[k]);
#pragma unroll
            for (int o = 0; o < OUT; o++) {
                float tv = valid ? tgt[row * TGT + o] : 0.f;
                const float sc = sNorm[N_SCL + o];
                if (sc > 0.f) tv = asinhf(tv / sc);
                tn[o] = valid ? (tv - sNorm[N_MUT + o]) / sNorm[N_SGT + o] : 0.f;
            }
        }
        cta_sync();
        // forward
        if (t == 0) mma_chain(tb + C_D1, smem_u32(sm + G_X), sImg + IMG_W1, INP, HID, false);
        if (!(ok = commit_and_wait(bar, phase, &sOk, t))) break;
        for (int q = 0; q < 4; q++) {
            float v[16];
            tmem_ld16(tmem_at(tb, 32 * warp, C_D1 + 16 * q), v);
            for (int i = 0; i < 16; i++) {
                const float z = v[i] + sBias[16 * q + i];
                v[i] = silu(z);
            }
            store_both(sm, G_H1, G_H1T, t, 16 * q, v);
        }
        cta_sync();
        if (t == 0) mma_chain(tb + C_D2, smem_u32(sm + G_H1), sImg + IMG_W2, HID, HID, false);
        if (!(ok = commit_and_wait(bar, phase, &sOk, t))) break;
        for (int q = 0; q < 4; q++) {
            float v[16];
            tmem_ld16(tmem_at(tb, 32 * warp, C_D2 + 16 * q), v);
            for (int i = 0; i < 16; i++) {
                const float z = v[i] + sBias[HID + 16 * q + i];
                v[i] = silu(z);
            }
            store_both(sm, G_H2, G_H2T, t, 16 * q, v);
        }
        cta_sync();
        if (t == 0) mma_chain(tb + C_D3, smem_u32(sm + G_H2), sImg + IMG_W3, HID, OUTP, false);
        if (!(ok = commit_and_wait(bar, phase, &sOk, t))) break;
        {
            float y[16], dy[16];
            tmem_ld16(tmem_at(tb, 32 * warp, C_D3), y);
            float l = 0.f;
#pragma unroll
            for (int o = 0; o < OUTP; o++) dy[o] = 0.f;
#pragma unroll
            for (int o = 0; o < OUT; o++) {
                const float e = valid ? y[o] + sBias[2 * HID + o] - tn[o] : 0.f;
                l += e * e;
                dy[o] = 2.f * e * invScale;
            }
            const float ls = warp_sum(l);
            if (lane == 0) sLoss[warp] += ls;
            store_row8(sm + G_Q, t, 0, OUTP, dy);
            store_row8(sm + G_Q, t, 8, OUTP, dy + 8);
#pragma unroll
            for (int o = 0; o < OUTP; o++) store_bf16(sm + G_P, core_off(o, t, TILE), dy[o]);
            bias_grad(dbRow, lane, 2 * HID, dy, OUT);
        }
        cta_sync();
        // backward: dH2 = dY W3, dW3 += dY^T H2
        if (t == 0) {
            mma_chain(tb + C_G2, smem_u32(sm + G_Q), sImg + IMG_W3T, OUTP, HID, false);
            mma_chain(tb + C_DW3, smem_u32(sm + G_P), smem_u32(sm + G_H2T), TILE, HID, j > 0);
        }
        if (!(ok = commit_and_wait(bar, phase, &sOk, t))) break;
        for (int q = 0; q < 4; q++) {
            float z[16], g[16];
            tmem_ld16(tmem_at(tb, 32 * warp, C_D2 + 16 * q), z);
            tmem_ld16(tmem_at(tb, 32 * warp, C_G2 + 16 * q), g);
            for (int i = 0; i < 16; i++) {
                const float a = z[i] + sBias[HID + 16 * q + i];
                g[i] *= silu_slope(a);
            }
            store_row8(sm + G_Q, t, 16 * q, HID, g);
            store_row8(sm + G_Q, t, 16 * q + 8, HID, g + 8);
            for (int i = 0; i < 16; i++) store_bf16(sm + G_P, core_off(16 * q + i, t, TILE), g[i]);
            bias_grad(dbRow, lane, HID + 16 * q, g, 16);
        }
        cta_sync();
        // dH1 = dZ2 W2, dW2 += dZ2^T H1
        if (t == 0) {
            mma_chain(tb + C_G1, smem_u32(sm + G_Q), sImg + IMG_W2T, HID, HID, false);
            mma_chain(tb + C_DW2, smem_u32(sm + G_P), smem_u32(sm + G_H1T), TILE, HID, j > 0);
        }
        if (!(ok = commit_and_wait(bar, phase, &sOk, t))) break;
        for (int q = 0; q < 4; q++) {
            float z[16], g[16];
            tmem_ld16(tmem_at(tb, 32 * warp, C_D1 + 16 * q), z);
            tmem_ld16(tmem_at(tb, 32 * warp, C_G1 + 16 * q), g);
            for (int i = 0; i < 16; i++) {
                const float a = z[i] + sBias[16 * q + i];
                g[i] *= silu_slope(a);
            }
            for (int i = 0; i < 16; i++) store_bf16(sm + G_P, core_off(16 * q + i, t, TILE), g[i]);
            bias_grad(dbRow, lane, 16 * q, g, 16);
        }
        cta_sync();
        // dW1 += dZ1^T X
        if (t == 0) mma_chain(tb + C_DW1, smem_u32(sm + G_P), smem_u32(sm + G_XT), TILE, INP, j > 0);
        if (!(ok = commit_and_wait(bar, phase, &sOk, t))) break;
    }
    if (ok) {
        float* dst = partial + (size_t)blockIdx.x * PARTIAL;
        if (warp < 2) {
            const int r = 32 * warp + lane;
            for (int q = 0; q < 2; q++) {
                float v[16];
                tmem_ld16(tmem_at(tb, 32 * warp, C_DW1 + 16 * q), v);
                for (int i = 0; i < 16; i++) dst[P_W1 + r * INP + 16 * q + i] = v[i];
            }
            for (int q = 0; q < 4; q++) {
                float v[16];
                tmem_ld16(tmem_at(tb, 32 * warp, C_DW2 + 16 * q), v);
                for (int i = 0; i < 16; i++) dst[P_W2 + r * HID + 16 * q + i] = v[i];
            }
        }
        if (warp == 0) {
            for (int q = 0; q < 4; q++) {
                float v[16];
                tmem_ld16(tmem_at(tb, 0, C_DW3 + 16 * q), v);
                if (lane < OUTP)
                    for (int i = 0; i < 16; i++) dst[P_W3 + lane * HID + 16 * q + i] = v[i];
            }
        }
        __syncthreads();
        for (int i = t; i < NBIAS; i += TILE)
            dst[P_B1 + i] = ((sDb[i] + sDb[NBIAS + i]) + sDb[2 * NBIAS + i]) + sDb[3 * NBIAS + i];
        if (t == 0) dst[NPARAM] = ((sLoss[0] + sLoss[1]) + sLoss[2]) + sLoss[3];
    }
    cta_sync();
    if (!sOk) drain(bar, phase, t, status);
    cta_sync();
    if (warp == 0) tmem_dealloc(tb, 512);
}

// ---------------------------------------------------------------------------
// Adam and the weight image
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pack_param(int p, float w, unsigned char* image, float* bias) {
    if (p < P_W2) {
        const int o = (p - P_W1) / INP, i = (p - P_W1) % INP;
        store_bf16(image, IMG_W1 + core_off(o, i, INP), w);
    } else if (p < P_W3) {
        const int o = (p - P_W2) / HID, i = (p - P_W2) % HID;
        store_bf16(image, IMG_W2 + core_off(o, i, HID), w);
        store_bf16(image, IMG_W2T + core_off(i, o, HID), w);
    } else if (p < P_B1) {
        const int o = (p - P_W3) / HID, i = (p - P_W3) % HID;
        store_bf16(image, IMG_W3 + core_off(o, i, HID), w);
        store_bf16(image, IMG_W3T + core_off(i, o, OUTP), w);
    } else {
        bias[p - P_B1] = w;
    }
}

__global__ void k_mlp_adam(int ctas, const float* __restrict__ partial, float* master, float* m1, float* m2,
                           float c1, float c2, float lr, int update, unsigned char* image, float* bias,
                           float* gradOut, float* lossOut) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == NPARAM && lossOut) {
        float l = 0.f;
        for (int c = 0; c < ctas; c++) l += partial[(size_t)c * PARTIAL + NPARAM];
        lossOut[0] = l;
    }
    if (p >= NPARAM) return;
    float g = 0.f;
    for (int c = 0; c < ctas; c++) g += partial[(size_t)c * PARTIAL + p];
    if (gradOut) gradOut[p] = g;
    float w = master[p];
    if (update) {
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        const float a = b1 * m1[p] + (1.f - b1) * g;
        const float v = b2 * m2[p] + (1.f - b2) * g * g;
        m1[p] = a;
        m2[p] = v;
        w -= lr * (a * c1) / (sqrtf(v * c2) + eps);
        master[p] = w;
    }
    pack_param(p, w, image, bias);
}

__global__ void k_mlp_pack(const float* __restrict__ master, unsigned char* image, float* bias) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NPARAM) pack_param(p, master[p], image, bias);
}

// ---------------------------------------------------------------------------
// Column statistics, targets, audit
// ---------------------------------------------------------------------------
constexpr int ST_THREADS = 256, ST_BLOCKS = 304, ST_MAXC = 24;

__global__ void __launch_bounds__(ST_THREADS) k_stats_partial(long long rows, int cols, int stride,
                                                             const float* __restrict__ data,
                                                             double* __restrict__ partial) {
    __shared__ double sh[ST_THREADS];
    double s[ST_MAXC], q[ST_MAXC];
    for (int c = 0; c < ST_MAXC; c++) s[c] = q[c] = 0.0;
    const long long per = (rows + gridDim.x - 1) / gridDim.x;
    const long long lo = per * blockIdx.x, hi = min(rows, lo + per);
    for (long long r = lo + threadIdx.x; r < hi; r += ST_THREADS)
        for (int c = 0; c < ST_MAXC; c++)
            if (c < cols) {
                const double v = data[r * stride + c];
                s[c] += v;
                q[c] += v * v;
            }
    for (int c = 0; c < 2 * cols; c++) {
        sh[threadIdx.x] = (c & 1) ? q[c >> 1] : s[c >> 1];
        __syncthreads();
        for (int w = ST_THREADS / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * 2 * ST_MAXC + c] = sh[0];
        __syncthreads();
    }
}

__global__ void k_stats_final(long long rows, int cols, int blocks, const double* __restrict__ partial,
                              double* __restrict__ out) {
    const int c = threadIdx.x;
    if (c >= cols) return;
    double s = 0.0, q = 0.0;
    for (int b = 0; b < blocks; b++) {
        s += partial[(size_t)b * 2 * ST_MAXC + 2 * c];
        q += partial[(size_t)b * 2 * ST_MAXC + 2 * c + 1];
    }
    const double mean = rows > 0 ? s / (double)rows : 0.0;
    const double var = rows > 0 ? fmax(q / (double)rows - mean * mean, 0.0) : 0.0;
    out[2 * c] = mean;
    out[2 * c + 1] = sqrt(var);
}

__global__ void k_target_transform(long long rows, const float* __restrict__ tgt, TargetScales sc,
                                   float* __restrict__ out) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
#pragma unroll
    for (int o = 0; o < OUT; o++) {
        const float t = tgt[r * TGT + o];
        out[r * TGT + o] = sc.s[o] > 0.f ? asinhf(t / sc.s[o]) : t;
    }
}

__global__ void k_targets(int n, const float4* __restrict__ refPos, const float4* __restrict__ refVel,
                          const float4* __restrict__ pos, const float4* __restrict__ vel, float* __restrict__ tgt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = refPos[i], b = pos[i], c = refVel[i], d = vel[i];
    float4* dst = reinterpret_cast<float4*>(tgt + (size_t)i * TGT);
    dst[0] = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, c.x - d.x);
    dst[1] = make_float4(c.y - d.y, c.z - d.z, 0.f, 0.f);
}

__global__ void k_audit(int n, const float* __restrict__ rhoA, const float* __restrict__ rhoB,
                        unsigned int* errBits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.f;
    if (i < n) {
        const float a = rhoA[i], b = rhoB[i];
        e = fabsf(a - b) / (b > 0.f ? b : 1.f);
        if (!(e == e)) e = __int_as_float(0x7F800000);  // NaN counts as an infinite error
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e = fmaxf(e, __shfl_xor_sync(0xFFFFFFFFu, e, o));
    if ((threadIdx.x & 31) == 0) atomicMax(errBits, __float_as_uint(e));
}

__global__ void k_audit_select(int n, const unsigned int* __restrict__ errBits, float tol,
                               const float4* __restrict__ srcPos, const float4* __restrict__ srcVel,
                               float4* __restrict__ pos, float4* __restrict__ vel, unsigned int* counters,
                               int* reuse) {
    const unsigned int bits = *errBits;
    const bool accept = __uint_as_float(bits) <= tol;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        counters[0] += 1;               // audits
        if (!accept) counters[1] += 1;  // rollbacks
        counters[2] = bits;             // last error
        counters[3] = max(counters[3], bits);
        if (reuse) *reuse = accept ? 1 : 0;
    }
    if (accept && i < n) {
        pos[i] = srcPos[i];
        vel[i] = srcVel[i];
    }
}

}  // namespace

void launch_mlp_apply(int n, const float* feat, MlpDev m, int mode, const int* workIds, float4* pos, float4* vel,
                      PhysDev ph, int collide, float* out, unsigned int* status, cudaStream_t s) {
    ensure_dynamic_smem<k_mlp_apply>(A_SMEM);
    const int tiles = (n + TILE - 1) / TILE;
    const int sms = device_sms();
    const int grid = tiles < A_CTAS_PER_SM * sms ? tiles : A_CTAS_PER_SM * sms;
    if (grid > 0)
        k_mlp_apply<<<grid, TILE, A_SMEM, s>>>(n, feat, m, mode, workIds, pos, vel, ph, collide, out, status);
}

void launch_mlp_grad(int ctas, int tilesPerCta, const int* tileList, const float* feat, const float* tgt,
                     long long count, float invScale, MlpDev m, float* partial, unsigned int* status,
                     cudaStream_t s) {
    ensure_dynamic_smem<k_mlp_grad>(G_SMEM);
    k_mlp_grad<<<ctas, TILE, G_SMEM, s>>>(tilesPerCta, tileList, feat, tgt, count, invScale, m, partial, status);
}

void launch_mlp_adam(int ctas, const float* partial, float* master, float* m1, float* m2, int t, float lr,
                     int update, unsigned char* image, float* bias, float* gradOut, float* lossOut,
                     cudaStream_t s) {
    const float c1 = t > 0 ? 1.f / (1.f - (float)std::pow(0.9, t)) : 1.f;
    const float c2 = t > 0 ? 1.f / (1.f - (float)std::pow(0.999, t)) : 1.f;
    k_mlp_adam<<<(NPARAM + 1 + 255) / 256, 256, 0, s>>>(ctas, partial, master, m1, m2, c1, c2, lr, update, image,
                                                        bias, gradOut, lossOut);
}

void launch_mlp_pack(const float* master, unsigned char* image, float* bias, cudaStream_t s) {
    k_mlp_pack<<<(NPARAM + 255) / 256, 256, 0, s>>>(master, image, bias);
}

void launch_column_stats(long long rows, int cols, int stride, const float* data, double* partial, double* out,
                         cudaStream_t s) {
    k_stats_partial<<<ST_BLOCKS, ST_THREADS, 0, s>>>(rows, cols, stride, data, partial);
    k_stats_final<<<1, 32, 0, s>>>(rows, cols, ST_BLOCKS, partial, out);
}

void launch_target_transform(long long rows, const float* tgt, TargetScales sc, float* out, cudaStream_t s) {
    if (rows > 0) k_target_transform<<<(unsigned int)((rows + 255) / 256), 256, 0, s>>>(rows, tgt, sc, out);
}

void launch_targets(int n, const float4* refPos, const float4* refVel, const float4* pos, const float4* vel,
                    float* tgt, cudaStream_t s) {
    k_targets<<<(n + 255) / 256, 256, 0, s>>>(n, refPos, refVel, pos, vel, tgt);
}

void launch_audit(int n, const float* rhoA, const float* rhoB, unsigned int* errBits, cudaStream_t s) {
    k_audit<<<(n + 255) / 256, 256, 0, s>>>(n, rhoA, rhoB, errBits);
}

void launch_audit_select(int n, const unsigned int* errBits, float tol, const float4* srcPos, const float4* srcVel,
                         float4* pos, float4* vel, unsigned int* counters, int* reuse, cudaStream_t s) {
    k_audit_select<<<(n + 255) / 256, 256, 0, s>>>(n, errBits, tol, srcPos, srcVel, pos, vel, counters, reuse);
}

}  // namespace sph
