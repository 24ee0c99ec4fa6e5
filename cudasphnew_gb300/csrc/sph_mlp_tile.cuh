// Device helpers of the corrector MLP's 128-row tiles, shared by the
// standalone kernels (sph_mlp.cu) and the learned step's fused force kernel
// (sph_step.cu): BF16 operand stores in the tensor-core layout, the
// commit -> mbarrier wait round trip with an iteration limit, the SiLU
// epilogue read from TMEM, and the decoding of the network's output.
#pragma once

#include "sph_corrector.h"
#include "sph_tc.cuh"

namespace sph {
namespace mlp {

constexpr uint32_t WAIT_LIMIT = 1u << 22;
constexpr float ASINH_1000 = 7.6009027f;  // asinh(1000) = ln(1000 + sqrt(1000001))

// tanh through the hardware approximation (tanh.approx.f32, relative error
// about 2^-11: below the BF16 rounding each activation gets next).
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// SiLU z sigmoid(z), with sigmoid(z) = (1 + tanh(z/2)) / 2: h + h tanh(h)
// for h = z/2.  One transcendental instead of an exponential and a division.
__device__ __forceinline__ float silu(float z) {
    const float h = 0.5f * z;
    return fmaf(h, tanh_fast(h), h);
}

// d SiLU / dz = s (1 + z (1 - s)) with s = sigmoid(z) from the same tanh.
__device__ __forceinline__ float silu_slope(float z) {
    const float s = fmaf(0.5f, tanh_fast(0.5f * z), 0.5f);
    return s * fmaf(z, 1.f - s, 1.f);
}

__device__ __forceinline__ void store_bf16(unsigned char* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// Eight consecutive columns k0..k0+7 of row r of an R x K operand.
__device__ __forceinline__ void store_row8(unsigned char* base, int r, int k0, int K, const float* v) {
    uint4 q;
    q.x = tc::pack_bf16x2(v[0], v[1]);
    q.y = tc::pack_bf16x2(v[2], v[3]);
    q.z = tc::pack_bf16x2(v[4], v[5]);
    q.w = tc::pack_bf16x2(v[6], v[7]);
    *reinterpret_cast<uint4*>(base + tc::core_off(r, k0, K)) = q;
}

// Standardises the 24 raw features in place: (f - mean) / deviation, with
// the inverse deviations stored (`norm` 16-byte aligned).
__device__ __forceinline__ void standardise(float* f, const float* norm) {
    const float4* mu = reinterpret_cast<const float4*>(norm + N_MUX);
    const float4* is = reinterpret_cast<const float4*>(norm + N_ISX);
#pragma unroll
    for (int c = 0; c < IN / 4; c++) {
        const float4 a = mu[c], b = is[c];
        f[4 * c + 0] = (f[4 * c + 0] - a.x) * b.x;
        f[4 * c + 1] = (f[4 * c + 1] - a.y) * b.y;
        f[4 * c + 2] = (f[4 * c + 2] - a.z) * b.z;
        f[4 * c + 3] = (f[4 * c + 3] - a.w) * b.w;
    }
}

// Row r of a K = 32 feature tile: the 24 raw features standardised, padded
// with zeros; an invalid row is all zeros.  (Standardised straight from
// `raw`: no copy of the raw values stays live.)
__device__ __forceinline__ void store_feature_row(unsigned char* x, int r, const float* raw, bool valid,
                                                  const float* norm) {
    float f[INP];
#pragma unroll
    for (int k = 0; k < INP; k++) f[k] = 0.f;
    if (valid) {
        const float4* mu = reinterpret_cast<const float4*>(norm + N_MUX);
        const float4* is = reinterpret_cast<const float4*>(norm + N_ISX);
#pragma unroll
        for (int c = 0; c < IN / 4; c++) {
            const float4 a = mu[c], b = is[c];
            f[4 * c + 0] = (raw[4 * c + 0] - a.x) * b.x;
            f[4 * c + 1] = (raw[4 * c + 1] - a.y) * b.y;
            f[4 * c + 2] = (raw[4 * c + 2] - a.z) * b.z;
            f[4 * c + 3] = (raw[4 * c + 3] - a.w) * b.w;
        }
    }
#pragma unroll
    for (int c = 0; c < INP / 8; c++) store_row8(x, r, 8 * c, INP, f + 8 * c);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Issued by thread 0: the MMAs of one group are already enqueued; commit and
// wait.  Every thread then synchronises; returns false when the wait gave up.
__device__ __forceinline__ bool commit_and_wait(uint64_t* bar, uint32_t& phase, int* sOk, int t) {
    if (t == 0) {
        tc::mma_commit(bar);
        if (!tc::mbar_wait(bar, phase, WAIT_LIMIT)) *sOk = 0;
    }
    phase ^= 1u;
    tc::cta_sync();
    return *sOk != 0;
}

// After a wait gave up: one more bounded wait for the group in flight.
__device__ __forceinline__ void drain(uint64_t* bar, uint32_t phase, int t, unsigned int* status) {
    if (t == 0) {
        atomicOr(status, STATUS_DEVICE_WAIT);
        tc::mbar_wait(bar, phase ^ 1u, WAIT_LIMIT);
    }
}

// Layer-1 and layer-2 biases as the epilogue below takes them: halved
// (the SiLU works on h = z/2, and 0.5 v + 0.5 b rounds to exactly half of
// v + b), the output bias as it is.
__device__ __forceinline__ float epilogue_bias(const float* bias, int k) {
    return k < 2 * HID ? 0.5f * bias[k] : bias[k];
}

// bias + SiLU of the 64 accumulator columns at TMEM address `acc` (this
// warp's 32 lanes, from its first column), stored as BF16 row r of `dst`
// (K = 64); `hbias` holds the halved biases (epilogue_bias), 16-byte aligned.
// Equal, bit for bit, to silu(acc + bias).
__device__ __forceinline__ void hidden_layer_out(uint32_t acc, const float* hbias, unsigned char* dst, int r) {
#pragma unroll 1
    for (int q = 0; q < 2; q++) {
        float v[32];
        tc::tmem_ld32(acc + 32 * q, v);
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const float4 b = reinterpret_cast<const float4*>(hbias + 32 * q)[c];
            const float h0 = fmaf(0.5f, v[4 * c], b.x), h1 = fmaf(0.5f, v[4 * c + 1], b.y);
            const float h2 = fmaf(0.5f, v[4 * c + 2], b.z), h3 = fmaf(0.5f, v[4 * c + 3], b.w);
            v[4 * c] = fmaf(h0, tanh_fast(h0), h0);
            v[4 * c + 1] = fmaf(h1, tanh_fast(h1), h1);
            v[4 * c + 2] = fmaf(h2, tanh_fast(h2), h2);
            v[4 * c + 3] = fmaf(h3, tanh_fast(h3), h3);
        }
#pragma unroll
        for (int c = 0; c < 4; c++) store_row8(dst, r, 32 * q + 8 * c, HID, v + 8 * c);
    }
}

// The correction from the network's standardised output y (+ the last
// bias): mean + deviation * y, or s * sinh(...) for a compressed target,
// cut at |correction| <= 1000 s (sinh grows exponentially, so an
// out-of-range prediction is cut there).
__device__ __forceinline__ void decode_correction(const float* norm, const float* bias3, const float* y, float* c) {
#pragma unroll
    for (int o = 0; o < OUT; o++) {
        c[o] = norm[N_MUT + o] + norm[N_SGT + o] * (y[o] + bias3[o]);
        const float sc = norm[N_SCL + o];
        if (sc > 0.f) c[o] = sc * sinhf(fminf(fmaxf(c[o], -ASINH_1000), ASINH_1000));
    }
}

}  // namespace mlp
}  // namespace sph
