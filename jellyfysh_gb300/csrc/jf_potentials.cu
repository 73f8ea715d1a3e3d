// jf_potentials.cu -- batched potentials: the reference's Potential.displacement / Potential.derivative
// (jellyfysh/potential/potential.py:153-253) for arrays of (velocity, separation, charges, potential change),
// one thread per element, FP64 with the reference's arithmetic (jf_device.cuh).
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "jf_engine.cuh"

namespace jf {

enum PotentialOp {
    kHardSphereDisplacement,
    kInversePowerDisplacement,
    kInversePowerDerivative,
    kLennardJonesDisplacement,
    kLennardJonesDerivative,
    kDisplacedDisplacement,
    kDisplacedDerivative,
    kBoundDisplacement,
    kBoundDerivative,
    kMergedDerivative,
    kCellBoundingDisplacement
};

struct PotentialArgs {
    int op;
    int64_t n;
    double p0, p1, p2;  // parameters of the potential
    int32_t i0, i1;
    MH mh;
    MIC mic;
    IP ip;
    const double *velocity, *separation, *charges, *potential_change;
    const double *bounds_upper, *bounds_lower;
    const int32_t *cell_separation, *direction;
    const double *speed, *charge_factor;
    double *out;
    int32_t *status;
};

__device__ inline int evaluate(const PotentialArgs &a, int64_t i, double &out) {
    double v[3], s[3];
    if (a.op != kCellBoundingDisplacement) {
        for (int k = 0; k < 3; ++k) {
            v[k] = a.velocity[3 * i + k];
            s[k] = a.separation[3 * i + k];
        }
    }
    int d;
    double speed, value;
    switch (a.op) {
    case kHardSphereDisplacement:
        return hs_displacement(a.p0, v, s, out);
    case kInversePowerDisplacement:
        JF_TRY(analyse_velocity(v, d, speed));
        JF_TRY(ip_std_displacement(a.ip, d, s, a.charges[2 * i], a.charges[2 * i + 1], a.potential_change[i], value));
        out = value / speed;
        return JFGPU_STATUS_OK;
    case kInversePowerDerivative:
        JF_TRY(analyse_velocity(v, d, speed));
        JF_TRY(ip_std_derivative(a.ip, d, s, a.charges[2 * i], a.charges[2 * i + 1], value));
        out = value * speed;
        return JFGPU_STATUS_OK;
    case kLennardJonesDisplacement:
    case kDisplacedDisplacement:
        JF_TRY(analyse_velocity(v, d, speed));
        JF_TRY(mh_std_displacement(a.mh, d, s, a.potential_change[i], value));
        out = value / speed;
        return JFGPU_STATUS_OK;
    case kLennardJonesDerivative:
    case kDisplacedDerivative:
        JF_TRY(analyse_velocity(v, d, speed));
        JF_TRY(mh_std_derivative(a.mh, d, s, value));
        out = value * speed;
        return JFGPU_STATUS_OK;
    case kBoundDisplacement: {
        JF_TRY(analyse_velocity(v, d, speed));
        double p[3];
        permute3(s, d, p);
        out = ipcb_x_displacement(a.p0 * a.charges[2 * i] * a.charges[2 * i + 1], p[0], p[1], p[2],
                                  a.potential_change[i], a.p1) / speed;
        return JFGPU_STATUS_OK;
    }
    case kBoundDerivative: {
        JF_TRY(analyse_velocity(v, d, speed));
        double p[3];
        permute3(s, d, p);
        out = ipcb_x_derivative(a.p0 * a.charges[2 * i] * a.charges[2 * i + 1], p[0], p[1], p[2]) * speed;
        return JFGPU_STATUS_OK;
    }
    case kMergedDerivative:
        JF_TRY(analyse_velocity(v, d, speed));
        out = mic_std_derivative(a.mic, a.p0, d, s, a.charges[2 * i], a.charges[2 * i + 1]) * speed;
        return JFGPU_STATUS_OK;
    case kCellBoundingDisplacement: {
        // cell_bounding_potential.py:155-238
        int cs = a.cell_separation[i], dir = a.direction[i];
        double factor = a.charge_factor ? a.charge_factor[i] : 1.0;
        double rate = factor > 0.0 ? a.bounds_upper[cs * 3 + dir] * factor : a.bounds_lower[cs * 3 + dir] * factor;
        double disp = rate > 0 ? a.potential_change[i] / rate : kInf;
        out = disp / a.speed[i];
        return JFGPU_STATUS_OK;
    }
    default:
        return JFGPU_STATUS_ASSERTION;
    }
}

__global__ void potential_kernel(PotentialArgs a) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double out = 0.0;
    int st = evaluate(a, i, out);
    a.out[i] = st ? NAN : out;
    if (a.status) a.status[i] = st;
}

static int launch(PotentialArgs &a, void *stream) {
    if (a.n < 0 || !a.out) return JFGPU_ERROR_ARGUMENT;
    if (a.n == 0) return JFGPU_OK;
    const int threads = 128;
    int64_t blocks = (a.n + threads - 1) / threads;
    potential_kernel<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

static PotentialArgs base_args(int op, const double *velocity, const double *separation, int64_t n, double *out,
                               int32_t *status) {
    PotentialArgs a;
    memset(&a, 0, sizeof(a));
    a.op = op;
    a.velocity = velocity;
    a.separation = separation;
    a.n = n;
    a.out = out;
    a.status = status;
    return a;
}


}  // namespace jf

using namespace jf;

extern "C" {

int jfgpu_hard_sphere_displacement(double radius, const double *velocity, const double *separation, int64_t n,
                                   double *out, int32_t *status, void *stream) {
    PotentialArgs a = base_args(kHardSphereDisplacement, velocity, separation, n, out, status);
    a.p0 = 4.0 * radius * radius;
    return launch(a, stream);
}

int jfgpu_inverse_power_displacement(double power, double prefactor, const double *velocity,
                                     const double *separation, const double *charges,
                                     const double *potential_change, int64_t n, double *out, int32_t *status,
                                     void *stream) {
    if (!charges || !potential_change) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kInversePowerDisplacement, velocity, separation, n, out, status);
    a.ip = ip_make(power, prefactor);
    a.charges = charges;
    a.potential_change = potential_change;
    return launch(a, stream);
}

int jfgpu_inverse_power_derivative(double power, double prefactor, const double *velocity, const double *separation,
                                   const double *charges, int64_t n, double *out, int32_t *status, void *stream) {
    if (!charges) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kInversePowerDerivative, velocity, separation, n, out, status);
    a.ip = ip_make(power, prefactor);
    a.charges = charges;
    return launch(a, stream);
}

int jfgpu_lennard_jones_displacement(double prefactor, double characteristic_length, const double *velocity,
                                     const double *separation, const double *potential_change, int64_t n,
                                     double *out, int32_t *status, void *stream) {
    if (!potential_change) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kLennardJonesDisplacement, velocity, separation, n, out, status);
    a.mh = make_lj(prefactor, characteristic_length);
    a.potential_change = potential_change;
    return launch(a, stream);
}

int jfgpu_lennard_jones_derivative(double prefactor, double characteristic_length, const double *velocity,
                                   const double *separation, int64_t n, double *out, int32_t *status,
                                   void *stream) {
    PotentialArgs a = base_args(kLennardJonesDerivative, velocity, separation, n, out, status);
    a.mh = make_lj(prefactor, characteristic_length);
    return launch(a, stream);
}

int jfgpu_displaced_even_power_displacement(double equilibrium_separation, int32_t power, double prefactor,
                                            const double *velocity, const double *separation,
                                            const double *potential_change, int64_t n, double *out,
                                            int32_t *status, void *stream) {
    if (!potential_change || power <= 0 || power % 2) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kDisplacedDisplacement, velocity, separation, n, out, status);
    a.mh = make_displaced(equilibrium_separation, power, prefactor);
    a.potential_change = potential_change;
    return launch(a, stream);
}

int jfgpu_displaced_even_power_derivative(double equilibrium_separation, int32_t power, double prefactor,
                                          const double *velocity, const double *separation, int64_t n,
                                          double *out, int32_t *status, void *stream) {
    if (power <= 0 || power % 2) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kDisplacedDerivative, velocity, separation, n, out, status);
    a.mh = make_displaced(equilibrium_separation, power, prefactor);
    return launch(a, stream);
}

int jfgpu_coulomb_bound_displacement(double prefactor, double system_length, const double *velocity,
                                     const double *separation, const double *charges,
                                     const double *potential_change, int64_t n, double *out, int32_t *status,
                                     void *stream) {
    if (!charges || !potential_change) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kBoundDisplacement, velocity, separation, n, out, status);
    a.p0 = prefactor;
    a.p1 = system_length;
    a.charges = charges;
    a.potential_change = potential_change;
    return launch(a, stream);
}

int jfgpu_coulomb_bound_derivative(double prefactor, const double *velocity, const double *separation,
                                   const double *charges, int64_t n, double *out, int32_t *status, void *stream) {
    if (!charges) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kBoundDerivative, velocity, separation, n, out, status);
    a.p0 = prefactor;
    a.charges = charges;
    return launch(a, stream);
}

int jfgpu_merged_image_coulomb_derivative(double alpha, int32_t fourier_cutoff, int32_t position_cutoff,
                                          double prefactor, double system_length, const double *velocity,
                                          const double *separation, const double *charges, int64_t n,
                                          double *out, int32_t *status, void *stream) {
    if (!charges || fourier_cutoff < 0 || position_cutoff < 0 || !(alpha > 0.0)) return JFGPU_ERROR_ARGUMENT;
    // Fourier coefficients (merged_image_coulomb_potential.c:77-119) on the host with the host libm
    int nf = fourier_cutoff + 1;
    size_t count = (size_t)nf * nf * nf;
    double *host = (double *)calloc(count, sizeof(double));
    if (!host) return JFGPU_ERROR_ALLOCATION;
    for (int k = 0; k < nf; k++)
        for (int j = 0; j < nf; j++)
            for (int i = 1; i < nf; i++) {
                double coefficient = (j == 0 && k == 0) ? 1.0 : ((k == 0 || j == 0) ? 2.0 : 4.0);
                double norm_sq = i * i + j * j + k * k;
                host[(i * nf + j) * nf + k] = 4.0 * i * coefficient / (norm_sq * system_length * system_length) *
                                              std::exp(-M_PI * M_PI * norm_sq / (alpha * alpha));
            }
    double *table = nullptr;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMallocAsync((void **)&table, count * sizeof(double), s) != cudaSuccess) {
        free(host);
        return JFGPU_ERROR_ALLOCATION;
    }
    int result = JFGPU_ERROR_CUDA;
    if (cudaMemcpyAsync(table, host, count * sizeof(double), cudaMemcpyHostToDevice, s) == cudaSuccess) {
        PotentialArgs a = base_args(kMergedDerivative, velocity, separation, n, out, status);
        a.p0 = prefactor;
        a.charges = charges;
        MIC m;
        m.fourier_cutoff = fourier_cutoff;
        m.fourier_cutoff_sq = fourier_cutoff * fourier_cutoff;
        m.position_cutoff = position_cutoff;
        m.position_cutoff_sq = position_cutoff * position_cutoff;
        m.alpha_over_length = alpha / system_length;
        m.alpha_over_length_sq = alpha * alpha / (system_length * system_length);
        m.two_alpha_over_length_root_pi = 2.0 * alpha / (system_length * std::sqrt(M_PI));
        m.system_length = system_length;
        m.two_pi_over_length = 2.0 * M_PI / system_length;
        m.fourier = table;
        a.mic = m;
        result = launch(a, stream);
    }
    cudaStreamSynchronize(s);  // the host table must outlive the copy
    free(host);
    cudaFreeAsync(table, s);
    return result;
}

int jfgpu_cell_bounding_displacement(const double *bounds_upper, const double *bounds_lower,
                                     const int32_t *cell_separation, const int32_t *direction, const double *speed,
                                     const double *charge_factor, const double *potential_change, int64_t n,
                                     double *out, int32_t *status, void *stream) {
    if (!bounds_upper || !cell_separation || !direction || !speed || !potential_change) return JFGPU_ERROR_ARGUMENT;
    if (charge_factor && !bounds_lower) return JFGPU_ERROR_ARGUMENT;
    PotentialArgs a = base_args(kCellBoundingDisplacement, nullptr, nullptr, n, out, status);
    a.bounds_upper = bounds_upper;
    a.bounds_lower = bounds_lower;
    a.cell_separation = cell_separation;
    a.direction = direction;
    a.speed = speed;
    a.charge_factor = charge_factor;
    a.potential_change = potential_change;
    return launch(a, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------------------
// The merged-image Coulomb derivative for callers that cannot allocate device memory.
//
// jfgpu_merged_image_coulomb_derivative allocates its Fourier-coefficient table with cudaMallocAsync on every call.
// Some callers cannot do that: hosts that must not enter the CUDA allocator once they are running (real-time loops,
// embedded controllers with a fixed memory budget), and plug-ins that live inside another framework whose memory
// pool owns the device.  For them the table lives in the file-scope device array below, of a fixed maximum size,
// which every GPU that loads this library keeps until the process exits, and is filled on the device by a small
// kernel from the parameters passed by value (no host buffer, no copy).  The caller still passes every input and
// output array.
// ---------------------------------------------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxFourierCutoff = 15;  // (15 + 1)^3 doubles = 32 KiB
constexpr int kNoAllocSide = kNoAllocMaxFourierCutoff + 1;
constexpr int kNoAllocEntries = kNoAllocSide * kNoAllocSide * kNoAllocSide;

__device__ __align__(256) double g_merged_image_fourier[kNoAllocEntries];

std::mutex g_fourier_mutex;
double *g_fourier_address[128] = {};  // device address of the array, per device ordinal

// In host code the array's name only stands for the symbol: the device address is looked up once per device,
// with that device current, and cached.
int fourier_scratch(double **address) {
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 128) return JFGPU_ERROR_CUDA;
    std::lock_guard<std::mutex> lock(g_fourier_mutex);
    if (!g_fourier_address[device]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_merged_image_fourier) != cudaSuccess || ptr == nullptr)
            return JFGPU_ERROR_CUDA;
        g_fourier_address[device] = static_cast<double *>(ptr);
    }
    *address = g_fourier_address[device];
    return JFGPU_OK;
}

// The Fourier coefficients of merged_image_coulomb_potential.c:77-119 in the table layout [i][j][k] of the cutoff,
// one thread per entry: every entry of the layout is written (the unused i = 0 plane as zeros), so nothing of an
// earlier call remains.  The device exp may differ from the host libm's by an ulp; the derivative then differs from
// the allocating entry point's at the 1e-16 relative level.
__global__ void fourier_table_kernel(double *table, int nf, double alpha, double system_length) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nf * nf * nf) return;
    const int i = e / (nf * nf), j = (e / nf) % nf, k = e % nf;
    double value = 0.0;
    if (i > 0) {
        const double coefficient = (j == 0 && k == 0) ? 1.0 : ((k == 0 || j == 0) ? 2.0 : 4.0);
        const double norm_sq = i * i + j * j + k * k;
        const double pi = 3.141592653589793;
        value = 4.0 * i * coefficient / (norm_sq * system_length * system_length) *
                exp(-pi * pi * norm_sq / (alpha * alpha));
    }
    table[e] = value;
}

}  // namespace

extern "C" int jfgpu_merged_image_coulomb_derivative_noalloc(double alpha, int32_t fourier_cutoff,
                                                             int32_t position_cutoff, double prefactor,
                                                             double system_length, const double *velocity,
                                                             const double *separation, const double *charges,
                                                             int64_t n, double *out, int32_t *status, void *stream) {
    if (!charges || !velocity || !separation || fourier_cutoff < 0 || position_cutoff < 0 || !(alpha > 0.0) ||
        !(system_length > 0.0))
        return JFGPU_ERROR_ARGUMENT;
    if (fourier_cutoff > kNoAllocMaxFourierCutoff) return JFGPU_ERROR_ARGUMENT;  // beyond the fixed table
    double *table = nullptr;
    int error = fourier_scratch(&table);
    if (error) return error;
    const int nf = fourier_cutoff + 1;
    const int count = nf * nf * nf;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    fourier_table_kernel<<<(count + 255) / 256, 256, 0, s>>>(table, nf, alpha, system_length);
    if (cudaGetLastError() != cudaSuccess) return JFGPU_ERROR_CUDA;
    PotentialArgs a = base_args(kMergedDerivative, velocity, separation, n, out, status);
    a.p0 = prefactor;
    a.charges = charges;
    MIC m;
    m.fourier_cutoff = fourier_cutoff;
    m.fourier_cutoff_sq = fourier_cutoff * fourier_cutoff;
    m.position_cutoff = position_cutoff;
    m.position_cutoff_sq = position_cutoff * position_cutoff;
    m.alpha_over_length = alpha / system_length;
    m.alpha_over_length_sq = alpha * alpha / (system_length * system_length);
    m.two_alpha_over_length_root_pi = 2.0 * alpha / (system_length * std::sqrt(M_PI));
    m.system_length = system_length;
    m.two_pi_over_length = 2.0 * M_PI / system_length;
    m.fourier = table;
    a.mic = m;
    return launch(a, stream);
}
