// Internal declarations of the learned step corrector: the per-particle MLP
// 24 -> 64 -> 64 -> 6 (SiLU) with BF16 weights and activations on tcgen05
// tensor cores (FP32 accumulation in TMEM) and its Adam trainer.  The
// features it reads are computed by the force stage (feature_values,
// sph_step.cu).  Not part of the public ABI.
#pragma once

#include "sph_internal.h"

namespace sph {

namespace mlp {

constexpr int IN = 24;     // features
constexpr int INP = 32;    // padded to the MMA's K granule
constexpr int HID = 64;
constexpr int OUT = 6;     // position and velocity correction
constexpr int OUTP = 16;   // padded to the smallest N of an M = 128 MMA
constexpr int TILE = 128;  // samples per CTA tile (the MMA's M)
constexpr int TGT = 8;     // floats per stored target (6 used)

// FP32 master parameters, in this order.
constexpr int P_W1 = 0;                     // [HID][INP]
constexpr int P_W2 = P_W1 + HID * INP;      // [HID][HID]
constexpr int P_W3 = P_W2 + HID * HID;      // [OUTP][HID]
constexpr int P_B1 = P_W3 + OUTP * HID;     // [HID]
constexpr int P_B2 = P_B1 + HID;            // [HID]
constexpr int P_B3 = P_B2 + HID;            // [OUTP]
constexpr int NPARAM = P_B3 + OUTP;         // 7312
constexpr int PARTIAL = NPARAM + 16;        // per-CTA gradient row (+ loss)

// Normalisation block: feature mean and inverse deviation, target mean and
// deviation, target scale.  With a scale s > 0 the network predicts the
// compressed target asinh(t/s) (standardised), so small and large corrections
// weigh alike; the correction is s*sinh(prediction).  s <= 0: t itself.
constexpr int N_MUX = 0, N_ISX = IN, N_MUT = 2 * IN, N_SGT = 2 * IN + OUT, N_SCL = 2 * IN + 2 * OUT, NNORM = 72;
constexpr int NSTATS = 2 * IN + 3 * OUT;  // host-side blob tail: means, deviations, scales

// BF16 weight image, byte offsets: the shared-memory layouts the kernels copy.
constexpr int IMG_W1 = 0;                  // W1  [64 x 32]
constexpr int IMG_W2 = 4096;               // W2  [64 x 64]
constexpr int IMG_W3 = 12288;              // W3  [16 x 64]
constexpr int IMG_W3T = 14336;             // W3^T [64 x 16]
constexpr int IMG_W2T = 16384;             // W2^T [64 x 64]
constexpr int IMG_BYTES = 24576;
constexpr int IMG_FWD_BYTES = 14336;       // W1, W2, W3: what inference needs
constexpr int NBIAS = HID + HID + OUTP;    // b1, b2, b3 (FP32)

}  // namespace mlp

// Device state of a corrector.
struct MlpDev {
    const unsigned char* image;  // IMG_BYTES
    const float* bias;           // NBIAS
    const float* norm;           // NNORM
};

// Inference over rows u < n.  mode 0: the features of particle id =
// workIds[u] (rows of `feat` in particle order), whose correction is added to
// pos/vel[id] (then collided when `collide`); mode 1: feature row u, and the
// correction (6 floats) is written to out[u].
void launch_mlp_apply(int n, const float* feat, MlpDev m, int mode, const int* workIds, float4* pos, float4* vel,
                      PhysDev ph, int collide, float* out, unsigned int* status, cudaStream_t s);

// One optimiser step's gradients: `ctas` CTAs, CTA c takes tiles
// tileList[c * tilesPerCta + j]; tile t covers samples t*128 .. t*128+127 of
// feat/tgt (rows >= count are padding).  Writes partial[c][PARTIAL].
void launch_mlp_grad(int ctas, int tilesPerCta, const int* tileList, const float* feat, const float* tgt,
                     long long count, float invScale, MlpDev m, float* partial, unsigned int* status,
                     cudaStream_t s);

// Sums the partial rows in order and applies Adam (step index t >= 1) to the
// master weights, then rewrites the BF16 image and the FP32 biases.
// gradOut (optional) receives the summed gradient, lossOut[0] the summed loss.
void launch_mlp_adam(int ctas, const float* partial, float* master, float* m1, float* m2, int t, float lr,
                     int update, unsigned char* image, float* bias, float* gradOut, float* lossOut,
                     cudaStream_t s);

// Rewrites the BF16 image and the FP32 biases from the master weights.
void launch_mlp_pack(const float* master, unsigned char* image, float* bias, cudaStream_t s);

// Per-column mean and deviation of rows of `cols` floats (stride `stride`),
// in double precision, deterministic: out[2*c] = mean, out[2*c+1] = deviation.
void launch_column_stats(long long rows, int cols, int stride, const float* data, double* partial, double* out,
                         cudaStream_t s);

// out[r] = asinh(tgt[r][o] / scale[o]) for the 6 components of `rows` targets
// (stride TGT in and out; a scale <= 0 copies the component).
struct TargetScales {
    float s[mlp::OUT];
};
void launch_target_transform(long long rows, const float* tgt, TargetScales sc, float* out, cudaStream_t s);

// Training targets: tgt[id] = (x_ref - x_coarse, v_ref - v_coarse, 0, 0).
void launch_targets(int n, const float4* refPos, const float4* refVel, const float4* pos, const float4* vel,
                    float* tgt, cudaStream_t s);

// Audit: err = max_i |rhoA_i - rhoB_i| / rhoB_i over particles (as float bits
// in *errBits, which must start at 0); then, when err <= tol, copies
// (srcPos, srcVel) over (pos, vel) and counts an acceptance, else a rollback.
void launch_audit(int n, const float* rhoA, const float* rhoB, unsigned int* errBits, cudaStream_t s);
// Keeps the learned result (srcPos, srcVel) when the audit error is within
// tol, else the plain one already in (pos, vel); *reuse = kept learned (the
// sorted copies, last made from the learned result, then hold the state).
void launch_audit_select(int n, const unsigned int* errBits, float tol, const float4* srcPos,
                         const float4* srcVel, float4* pos, float4* vel, unsigned int* counters, int* reuse,
                         cudaStream_t s);

// The learned step's force stage with the MLP fused in (sph_step.cu): the
// pretested pair loop (the density stage must have recorded the masks), or
// with `lists` the reused lists' exact masks (the list density stage must
// have run), wall terms, integration and collision, the features, the
// correction and one write-back; the raw features also go to feat.feat when
// it is set.
void launch_force_learned(int n, const float4* posS, const float4* velS, const float4* rho4S, const int* workIds,
                          RowTables T, GridDev g, PhysDev ph, MapDev map, int collide, const int* rowStart,
                          const unsigned int* rowMask, float4* pos, float4* vel, float4* accS, const StepConfig& cfg,
                          const FeatureOut& feat, MlpDev m, unsigned int* status, cudaStream_t s,
                          const NeighbourLists* lists = nullptr);

}  // namespace sph
