// jf_observe.cu -- observables of the chains' current configurations, for the estimators of long runs.
//
// One block per chain over all ordered pairs (i, j != i) of its units, with minimum-image separations as
// HypercubicPeriodicBoundaries.separation_vector (hypercubic_setting.py:120-140) takes them, from the FP32 mirror:
//   * the potential energy of the chain's pair potential: Lennard-Jones k s^12 / r^12 - k s^6 / r^6
//     (lennard_jones_potential.py:83-98), 0 for hard spheres; the merged-image Coulomb potential defines no
//     energy in the reference (only its derivative), so Coulomb chains report NaN;
//   * a histogram of the pair distances in [0, r_max), the pair-separation samples of the reference's
//     separation output handler (separation_output_handler.py:75-97) reduced to distances.
// Each unordered pair is met twice: the energy is halved and the shared-memory counts are even and halved.
// The estimators need no more than FP32 pair terms: they are summed per row in FP32 and across rows in FP64.
#include <cuda_runtime.h>

#include "jf_engine.cuh"

namespace jf {

constexpr int kObserveThreads = 256;
constexpr int kObserveStage = 2048;  // units staged in shared memory (16 bytes each)

__global__ void __launch_bounds__(kObserveThreads) observe_kernel(EngineView view, long long first,
                                                                  const float4 *positions32, int bins, float r_max,
                                                                  double *energy, unsigned long long *histogram) {
    extern __shared__ unsigned char smem[];
    __shared__ double partial[kObserveThreads / 32];
    const long long c = first + blockIdx.x;
    const ChainDev &ch = view.chains[c];
    const SpeciesDev &sp = view.species[ch.species];
    const int n = ch.n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned int *hist = reinterpret_cast<unsigned int *>(smem);
    float4 *staged = reinterpret_cast<float4 *>(smem + ((size_t)bins * 4 + 15) / 16 * 16);
    const bool use_stage = n <= kObserveStage;
    for (int k = tid; k < bins; k += kObserveThreads) hist[k] = 0;
    if (use_stage)
        for (int i = tid; i < n; i += kObserveThreads) staged[i] = positions32[ch.pos_off + i];
    __syncthreads();
    const float4 *P = use_stage ? staged : positions32 + ch.pos_off;
    const float L = ch.L32, half = ch.half32;
    const float r_max_sq = r_max * r_max, inv_bin = (float)bins / r_max;
    const bool lj = ch.potential == JFGPU_POT_LENNARD_JONES;
    const float a12 = sp.lj32[0], a6 = sp.lj32[1];
    double total = 0.0;
    // warp w takes the row tiles w, w + 8, ...: lane = row, all lanes read the same column unit
    const int tiles = (n + 31) / 32;
    for (int tile = warp; tile < tiles; tile += kObserveThreads / 32) {
        const int i = tile * 32 + lane;
        const bool row = i < n;
        const float4 pi = row ? P[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float row_energy = 0.0f;
        for (int j = 0; j < n; ++j) {
            const float4 pj = P[j];
            if (!row || j == i) continue;
            float s[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (s[k] >= half) s[k] -= L;
                if (s[k] < -half) s[k] += L;
            }
            const float r2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
            if (lj) {
                const float ir2 = 1.0f / r2;
                const float ir6 = ir2 * ir2 * ir2;
                row_energy += (a12 * ir6 + a6) * ir6;
            }
            if (r2 < r_max_sq) {
                int bin = (int)(sqrtf(r2) * inv_bin);
                if (bin >= bins) bin = bins - 1;
                atomicAdd(hist + bin, 1u);
            }
        }
        total += (double)row_energy;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
    if (lane == 0) partial[warp] = total;
    __syncthreads();
    if (tid == 0 && energy) {
        double sum = 0.0;
        for (int w = 0; w < kObserveThreads / 32; ++w) sum += partial[w];
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        energy[blockIdx.x] = ch.potential == JFGPU_POT_COULOMB ? nan : 0.5 * sum;
    }
    if (histogram)
        for (int k = tid; k < bins; k += kObserveThreads)
            histogram[(long long)blockIdx.x * bins + k] += hist[k] / 2;
}

size_t observe_shared_bytes(int bins, int max_n) {
    size_t bytes = ((size_t)bins * 4 + 15) / 16 * 16;
    if (max_n <= kObserveStage) bytes += (size_t)max_n * 16;
    return bytes;
}

cudaError_t launch_observe(const EngineView &view, long long first, long long count, int max_n,
                           const float4 *positions32, int bins, double r_max, double *energy,
                           unsigned long long *histogram, const LaunchPlan &plan) {
    const size_t smem = observe_shared_bytes(bins, max_n);
    if (smem > 32 * 1024) {  // with the static reduction buffer, above the default 48 KB per block
        cudaError_t err = cudaFuncSetAttribute(observe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
        if (err != cudaSuccess) return err;
    }
    if (plan.clock) plan.clock->begin(plan.stream);
    observe_kernel<<<(unsigned)count, kObserveThreads, smem, plan.stream>>>(view, first, positions32, bins,
                                                                          (float)r_max, energy, histogram);
    if (plan.clock) plan.clock->end(plan.stream, JFGPU_KERNEL_OBSERVE);
    return cudaGetLastError();
}

}  // namespace jf
