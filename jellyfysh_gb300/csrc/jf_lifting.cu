// jf_lifting.cu -- batched lifting schemes: one thread per table (tables of composite objects hold a few units,
// e.g. 2 x 3 for two water molecules), the decision of jf_lifting.cuh.
#include <cuda_runtime.h>

#include "jf_lifting.cuh"

namespace jf {

struct LiftingArgs {
    int scheme, draw_mode;
    int64_t n;
    const double *rates;
    const int32_t *active;
    const int64_t *offsets;
    const double *draws;
    int64_t *selected;
    double *bound;
    int32_t *status;
};

__global__ void lifting_kernel(LiftingArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int64_t begin = a.offsets[i], end = a.offsets[i + 1];
    int64_t selected = -1;
    double bound = NAN;
    int st = JFGPU_STATUS_ASSERTION;  // offsets that decrease: no table
    if (end >= begin)
        st = lifting_select(a.scheme, a.draw_mode, a.rates + begin, a.active + begin, end - begin, a.draws[i],
                            selected, bound);
    a.selected[i] = selected;
    if (a.bound) a.bound[i] = bound;
    a.status[i] = st;
}

}  // namespace jf

extern "C" int jfgpu_lifting(int32_t scheme, int32_t draw_mode, const double *rates, const int32_t *active,
                             const int64_t *offsets, int64_t n, const double *draws, int64_t *selected,
                             double *bound, int32_t *status, void *stream) {
    if (scheme < JFGPU_LIFTING_INSIDE_FIRST || scheme > JFGPU_LIFTING_RATIO) return JFGPU_ERROR_ARGUMENT;
    if (draw_mode != JFGPU_DRAW_VALUE && draw_mode != JFGPU_DRAW_UNIT) return JFGPU_ERROR_ARGUMENT;
    if (n < 0) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;  // no table: every pointer may be null
    if (!rates || !active || !offsets || !draws || !selected || !status) return JFGPU_ERROR_ARGUMENT;
    jf::LiftingArgs a{scheme, draw_mode, n, rates, active, offsets, draws, selected, bound, status};
    const int threads = 128;
    const int64_t blocks = (n + threads - 1) / threads;
    jf::lifting_kernel<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}
