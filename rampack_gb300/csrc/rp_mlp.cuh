// Learned neighbour ordering: a 13 -> 64 -> 64 -> 1 ReLU network (BF16 weights, FP32
// accumulation) that scores, from a pair's relative position and orientation, how likely
// the pair is to overlap after a random move of the first particle.  It only orders exact
// tests: the sweep pre-tests each mover's best-ranked partners and short-circuits on a
// certain overlap; every decision is still the exact test's.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace rp {

constexpr int MLP_IN = 16;   // 13 features, zero-padded to one MMA k-tile
constexpr int MLP_H = 64;
constexpr int MLP_FEATURES = 13;
constexpr int MLP_PARTNERS = 2;  // partners pre-tested per move

// Parameter offsets (floats) in the FP32 master vector; BF16 copies use the same offsets.
constexpr int MLP_W1 = 0;                           // [64][16] row o, col i
constexpr int MLP_B1 = MLP_W1 + MLP_H * MLP_IN;     // [64]
constexpr int MLP_W2 = MLP_B1 + MLP_H;              // [64][64] row o, col i
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;      // [64]
constexpr int MLP_W3 = MLP_B2 + MLP_H;              // [64]
constexpr int MLP_B3 = MLP_W3 + MLP_H;              // [1]
constexpr int MLP_NPARAM = MLP_B3 + 1;              // 5313

// Features of the pair (i, j): d = p_j - p_i (in units of the interaction range), the two
// unit axes, |d|^2, a_i.a_j, d.a_i, d.a_j; three zeros pad to 16.
__host__ __device__ __forceinline__ void mlp_features(float3 d, float3 ai, float3 aj, float inv_range, float *f) {
    float dx = d.x * inv_range, dy = d.y * inv_range, dz = d.z * inv_range;
    f[0] = dx;
    f[1] = dy;
    f[2] = dz;
    f[3] = ai.x;
    f[4] = ai.y;
    f[5] = ai.z;
    f[6] = aj.x;
    f[7] = aj.y;
    f[8] = aj.z;
    f[9] = dx * dx + dy * dy + dz * dz;
    f[10] = ai.x * aj.x + ai.y * aj.y + ai.z * aj.z;
    f[11] = dx * ai.x + dy * ai.y + dz * ai.z;
    f[12] = dx * aj.x + dy * aj.y + dz * aj.z;
    f[13] = 0.f;
    f[14] = 0.f;
    f[15] = 0.f;
}

// Features of a pair of rigid bodies (polyspheres, polyspherocylinders), whose bend makes
// the whole orientation matter: with R_i, R_j the row-major orientations and d = p_j - p_i
// (in units of the interaction range), the separation in the body frame of i,
// b = R_i^T d, the primary (z) and secondary (x) axes of j in that frame, z' = R_i^T z_j and
// x' = R_i^T x_j, |b|^2, b.z', b.x' and the squared separation across i's primary axis
// b_x^2 + b_y^2; three zeros pad to 16.
__host__ __device__ __forceinline__ void mlp_features_body(float3 d, const float *ri, const float *rj, float inv_range,
                                                           float *f) {
    const float dx = d.x * inv_range, dy = d.y * inv_range, dz = d.z * inv_range;
    const float bx = ri[0] * dx + ri[3] * dy + ri[6] * dz;
    const float by = ri[1] * dx + ri[4] * dy + ri[7] * dz;
    const float bz = ri[2] * dx + ri[5] * dy + ri[8] * dz;
    const float zx = ri[0] * rj[2] + ri[3] * rj[5] + ri[6] * rj[8];
    const float zy = ri[1] * rj[2] + ri[4] * rj[5] + ri[7] * rj[8];
    const float zz = ri[2] * rj[2] + ri[5] * rj[5] + ri[8] * rj[8];
    const float xx = ri[0] * rj[0] + ri[3] * rj[3] + ri[6] * rj[6];
    const float xy = ri[1] * rj[0] + ri[4] * rj[3] + ri[7] * rj[6];
    const float xz = ri[2] * rj[0] + ri[5] * rj[3] + ri[8] * rj[6];
    f[0] = bx;
    f[1] = by;
    f[2] = bz;
    f[3] = zx;
    f[4] = zy;
    f[5] = zz;
    f[6] = xx;
    f[7] = xy;
    f[8] = xz;
    f[9] = bx * bx + by * by + bz * bz;
    f[10] = bx * zx + by * zy + bz * zz;
    f[11] = bx * xx + by * xy + bz * xz;
    f[12] = bx * bx + by * by;
    f[13] = 0.f;
    f[14] = 0.f;
    f[15] = 0.f;
}

struct MlpDev {
    const float *w32;            // FP32 master parameters
    const __nv_bfloat16 *w16;    // BF16 copies (the weights the network computes with)
};

}  // namespace rp
