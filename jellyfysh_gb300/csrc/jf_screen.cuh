// jf_screen.cuh -- FP32 screening solves of the mixed-precision event loop.
//
// Each function returns the candidate's time displacement in FP32 and raises `flag` when the FP32 value cannot
// be trusted to a relative error of about 2^-13 plus the absolute margin of the chain (near-tangent motion,
// cancellation near the Lennard-Jones minimum or near U + du = 0, branch decisions within rounding of their
// boundary, negative radicands).  Flagged candidates are always re-solved in FP64; the others are re-solved
// when they lie within the screening margin of the smallest FP32 time.
#pragma once
#include "jf_device.cuh"

namespace jf {

constexpr float kScreenRel = 1.0f / 4096.0f;  // conditioning thresholds
constexpr float kInf32 = __builtin_inff();

// solve paths of a candidate as the FP32 screening takes them; the FP64 re-solves are queued by path so that the
// threads of a warp follow one branch of the reference's case analysis
constexpr int kPathFrontOutside = 0;   // Lennard-Jones: in front, outside the minimum shell
constexpr int kPathBehindShell = 1;    // behind, outside, the line of motion crosses the shell
constexpr int kPathBehindNoShell = 2;  // behind, outside, the line misses the shell
constexpr int kPathFrontInside = 3;    // in front, inside the shell
constexpr int kPathBehindInside = 4;   // behind, inside the shell
constexpr int kPathHardSphere = 5;
constexpr int kPathFar = 6;            // far-field (cell-bounding) candidate
constexpr int kPaths = 7;

// potential change of a keyed draw in FP32 without FP64 instructions: the uniform is (bits >> 11) 2^-53; its top 32
// bits k give u within 2^-32, so -log1p(-u) (u < 1/2) and -log(1 - u) with 1 - u from 2^32 - k (u >= 1/2) carry a
// relative error of about 2^-22 except for u < 2^-16 or 1 - u < 2^-16, which are flagged
__device__ inline float expovariate32(uint64_t bits, float inv_beta, bool &flag) {
    const uint32_t k = (uint32_t)(bits >> 32);
    float du;
    if (k < 0x80000000u) {
        if (k < 0x10000u) flag = true;
        du = -log1pf(-(float)k * (1.0f / 4294967296.0f));
    } else {
        const uint32_t complement = 0u - k;  // 2^32 - k
        if (complement < 0x10000u) flag = true;
        du = -logf((float)complement * (1.0f / 4294967296.0f));
    }
    if (!(du >= 0.0f) || isinf(du)) flag = true;
    return du * inv_beta;
}

// minimum-image separation in FP32 from the FP32 mirror; flags components within rounding of +-L/2
__device__ inline void separation32(const float4 &a, const float4 &b, float L, float half, float margin, float *s,
                                    bool &flag) {
    float v[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float x = v[k];
        if (x >= half) x -= L;
        if (x < -half) x += L;
        if (fabsf(fabsf(x) - half) < margin) flag = true;
        s[k] = x;
    }
}

// hard sphere: t = (s^2 - d^2) / (v s_d + sqrt((v s_d)^2 - v^2 (s^2 - d^2))) / v, stable form
__device__ inline float hs_screen(float diameter_sq, int d, float speed, const float *s, float margin, bool &flag) {
    float sd = s[d];
    if (fabsf(sd) < margin) flag = true;
    if (sd < 0.0f) return kInf32;
    float s2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    float excess = s2 - diameter_sq;
    float disc = sd * sd - excess;
    float tol = kScreenRel * (sd * sd + diameter_sq);
    if (fabsf(disc) < tol || fabsf(excess) < tol) flag = true;
    if (disc < 0.0f) return kInf32;
    float root = sqrtf(disc);
    if (sd < 0.0625f * sqrtf(s2)) flag = true;  // near-tangent motion
    return (excess / (sd + root)) / speed;
}

// Lennard-Jones constants for the screening
struct LJ32 {
    float a12, a6;        // k sigma^12, -k sigma^6
    float four_over_k;    // 4 / k
    float sigma_sq;
    float r0_sq;
};

__device__ inline float lj_u32(const LJ32 &c, float norm_sq) {
    float ir2 = 1.0f / norm_sq;
    float ir6 = ir2 * ir2 * ir2;
    return (c.a12 * ir6 + c.a6) * ir6;
}

// squared radius where U = potential inside (sign = +1) or outside (sign = -1) the minimum:
// sigma^6 / r^6 = (1 +- sqrt(1 + 4U/k)) / 2
__device__ inline float lj_invert_sq32(const LJ32 &c, float potential, float sign, bool &flag) {
    float y = c.four_over_k * potential;
    float one_plus = 1.0f + y;
    if (one_plus < 1.0f / 256.0f) flag = true;  // close to the minimum: cancellation
    if (one_plus < 0.0f) {
        flag = true;
        one_plus = 0.0f;
    }
    float root = sqrtf(one_plus);
    float x = sign > 0.0f ? 0.5f * (1.0f + root) : (-0.5f * y) / (1.0f + root);
    if (!(x > 0.0f)) {
        flag = true;
        return kInf32;
    }
    // r^2 = sigma^2 x^(-1/3)
    return c.sigma_sq * exp2f(-__log2f(x) * (1.0f / 3.0f));
}

// s_d +- sqrt(r_new^2 - perp^2) with flags on small or negative radicands
__device__ inline float lj_disp32(float sd, float perp, float norm_sq_new, float sign, bool &flag) {
    float radicand = norm_sq_new - perp;
    if (radicand < kScreenRel * 16.0f * norm_sq_new) flag = true;
    if (radicand < 0.0f) return kInf32;
    return sign > 0.0f ? sd - sqrtf(radicand) : sd + sqrtf(radicand);
}

__device__ inline bool near32(float a, float b) { return fabsf(a - b) <= kScreenRel * (fabsf(a) + fabsf(b)); }

// front of the target and outside the minimum shell: climb from U
__device__ inline float lj_front_outside32(const LJ32 &c, float u, float du, float sd, float perp, bool &flag) {
    float target = u + du;
    if (near32(u, -du)) flag = true;
    if (target >= 0.0f) return kInf32;
    float nsq = lj_invert_sq32(c, target, -1.0f, flag);
    if (isinf(nsq)) return kInf32;
    return lj_disp32(sd, perp, nsq, -1.0f, flag);
}

// front and inside: slide to the shell, then climb
__device__ inline float lj_front_inside32(const LJ32 &c, float du, float sd, float perp, bool &flag) {
    float radicand = c.r0_sq - perp;
    if (radicand < kScreenRel * 16.0f * c.r0_sq) flag = true;
    if (radicand < 0.0f) {
        flag = true;
        return kInf32;
    }
    float disp = sd + sqrtf(radicand);
    float sd_new = sd - disp;
    float u = lj_u32(c, sd_new * sd_new + perp);
    return disp + lj_front_outside32(c, u, du, sd_new, perp, flag);
}

// behind and inside: climb to the maximum at s_d = 0 or pass it and continue in front
__device__ inline float lj_behind_inside32(const LJ32 &c, float u, float du, float sd, float perp, bool &flag) {
    float u_max = lj_u32(c, perp);
    float difference = u_max - u;
    if (near32(du, difference)) flag = true;
    if (du < difference) {
        float nsq = lj_invert_sq32(c, u + du, 1.0f, flag);
        return lj_disp32(sd, perp, nsq, 1.0f, flag);
    }
    return sd + lj_front_inside32(c, du - difference, 0.0f, perp, flag);
}

__device__ inline float lj_screen(const LJ32 &c, int d, float speed, const float *s, float du, float margin,
                                  bool &flag, int &path) {
    float sd = s[d];
    int a = d == 0 ? 1 : 0;
    int b = d == 2 ? 1 : 2;
    float perp = s[a] * s[a] + s[b] * s[b];
    float norm_sq = sd * sd + perp;
    if (fabsf(sd) < margin) flag = true;
    if (fabsf(norm_sq - c.r0_sq) < kScreenRel * c.r0_sq) flag = true;
    float disp;
    if (norm_sq >= c.r0_sq) {
        if (sd <= 0.0f) {
            path = kPathFrontOutside;
            disp = lj_front_outside32(c, lj_u32(c, norm_sq), du, sd, perp, flag);
        } else {
            // behind and outside: reach the shell if the line crosses it, else slide to s_d = 0
            float radicand = c.r0_sq - perp;
            if (fabsf(radicand) < kScreenRel * 16.0f * c.r0_sq) flag = true;
            if (radicand >= 0.0f) {
                path = kPathBehindShell;
                float to_shell = sd - sqrtf(radicand);
                float sd_new = sd - to_shell;
                float u = lj_u32(c, sd_new * sd_new + perp);
                disp = to_shell + lj_behind_inside32(c, u, du, sd_new, perp, flag);
            } else {
                path = kPathBehindNoShell;
                disp = sd + lj_front_outside32(c, lj_u32(c, perp), du, 0.0f, perp, flag);
            }
        }
    } else {
        if (sd <= 0.0f) {
            path = kPathFrontInside;
            disp = lj_front_inside32(c, du, sd, perp, flag);
        } else {
            path = kPathBehindInside;
            disp = lj_behind_inside32(c, lj_u32(c, norm_sq), du, sd, perp, flag);
        }
    }
    if (isnan(disp)) {
        flag = true;
        return 0.0f;
    }
    return disp / speed;
}

}  // namespace jf
