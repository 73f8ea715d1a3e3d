// jf_composite.cu -- batched events between two composite objects: one thread per event (a few units per object,
// each pair one merged-image Coulomb derivative), the arithmetic of jf_composite.cuh.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "jf_composite.cuh"
#include "jf_engine.cuh"

namespace jf {

struct CompositeArgs {
    CompositeModel model;
    int draw_mode;
    int64_t n;
    const double *velocity, *active_position, *active_charge, *target_positions, *target_charges;
    const double *potential_changes, *local_positions, *local_charges, *draws;
    const double *bounding_rates;  // given bounding event rates (molecular cell-bounding / cell-veto handlers), or null
    const int32_t *active_index, *local_first;
    double *displacement, *rates;
    int32_t *new_active, *status;
};

__global__ void composite_time_kernel(CompositeArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int k = a.model.units;
    double v[3], p[3];
    for (int c = 0; c < 3; ++c) {
        v[c] = a.velocity[3 * i + c];
        p[c] = a.active_position[3 * i + c];
    }
    double out = 0.0;
    const int st = composite_event_time(a.model, v, p, a.active_charge[i], a.target_positions + 3 * k * i,
                                        a.target_charges + k * i, a.potential_changes + k * i, out);
    a.displacement[i] = st ? NAN : out;
    a.status[i] = st;
}

__global__ void composite_out_kernel(CompositeArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int k = a.model.units;
    double v[3];
    for (int c = 0; c < 3; ++c) v[c] = a.velocity[3 * i + c];
    int new_active = -1;
    double bounding_rate = NAN, event_rate = NAN;
    const int active = a.active_index[i];
    int st = JFGPU_STATUS_ASSERTION;  // an active index outside the local object
    if (active >= 0 && active < k)
        st = composite_out_state(a.model, a.draw_mode, v, a.local_positions + 3 * k * i, a.local_charges + k * i,
                                 active, a.target_positions + 3 * k * i, a.target_charges + k * i,
                                 a.local_first[i], a.draws + 3 * i, new_active, bounding_rate, event_rate,
                                 a.bounding_rates ? a.bounding_rates + i : nullptr);
    a.new_active[i] = st ? -1 : new_active;
    if (a.rates) {
        a.rates[2 * i] = bounding_rate;
        a.rates[2 * i + 1] = event_rate;
    }
    a.status[i] = st;
}

struct CellTimeArgs {
    const double *upper, *lower;                // [cells][3]
    const double *walker_upper, *walker_lower;  // [3] (cell veto)
    int64_t cells, n;
    const int32_t *relative_cell;
    const double *velocity, *active_charge, *target_charges, *potential_change;
    int units;
    double dipole_charge;
    double *rate, *time;
    int32_t *status;
};

// one thread per event: the molecular cell-bounding (veto = false) or cell-veto event time
__global__ void cell_time_kernel(CellTimeArgs a, bool veto) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int32_t cell = a.relative_cell[i];
    double rate = NAN, time = NAN;
    int st = JFGPU_STATUS_INDEX;  // a relative cell outside the table
    if (cell >= 0 && cell < a.cells) {
        const double *v = a.velocity + 3 * i;
        st = veto ? composite_cell_veto_time(a.upper + 3 * cell, a.lower + 3 * cell, a.walker_upper, a.walker_lower,
                                             v, a.active_charge[i], a.potential_change[i], rate, time)
                  : composite_cell_bound_time(a.upper + 3 * cell, a.lower + 3 * cell, v, a.active_charge[i],
                                              a.target_charges + (int64_t)a.units * i, a.units, a.dipole_charge,
                                              a.potential_change[i], rate, time);
    }
    a.rate[i] = st ? NAN : rate;
    a.time[i] = st ? NAN : time;
    a.status[i] = st;
}

// the model with its Fourier table copied to the device on the caller's stream; the table is freed (stream-ordered)
// after the launch
static int make_model(const JfgpuCompositeDesc *desc, cudaStream_t stream, CompositeModel &m, double **table) {
    if (!desc || desc->units < 1 || desc->units > kMaxCompositeUnits) return JFGPU_ERROR_ARGUMENT;
    if (desc->lifting < JFGPU_LIFTING_INSIDE_FIRST || desc->lifting > JFGPU_LIFTING_RATIO) return JFGPU_ERROR_ARGUMENT;
    if (desc->fourier_cutoff < 0 || desc->position_cutoff < 0 || !(desc->alpha > 0.0) ||
        !(desc->system_length > 0.0))
        return JFGPU_ERROR_ARGUMENT;
    std::vector<double> host = fourier_table(desc->fourier_cutoff, desc->alpha, desc->system_length);
    if (cudaMallocAsync((void **)table, host.size() * sizeof(double), stream) != cudaSuccess)
        return JFGPU_ERROR_ALLOCATION;
    if (cudaMemcpyAsync(*table, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice, stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess) {  // the host table must outlive the copy
        cudaFreeAsync(*table, stream);
        return JFGPU_ERROR_CUDA;
    }
    m.mic = make_mic(desc->fourier_cutoff, desc->position_cutoff, desc->alpha, desc->system_length, *table);
    m.coulomb_prefactor = desc->coulomb_prefactor;
    m.bound_prefactor = desc->bound_prefactor;
    m.system_length = desc->system_length;
    m.units = desc->units;
    m.lifting = desc->lifting;
    return JFGPU_OK;
}

static int run(CompositeArgs &a, const JfgpuCompositeDesc *desc, void *stream, bool out_state) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *table = nullptr;
    int error = make_model(desc, s, a.model, &table);
    if (error) return error;
    const int threads = 64;
    const int64_t blocks = (a.n + threads - 1) / threads;
    if (out_state)
        composite_out_kernel<<<(unsigned)blocks, threads, 0, s>>>(a);
    else
        composite_time_kernel<<<(unsigned)blocks, threads, 0, s>>>(a);
    error = cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
    cudaFreeAsync(table, s);
    return error;
}

}  // namespace jf

extern "C" int jfgpu_composite_event_time(const JfgpuCompositeDesc *desc, const double *velocity,
                                          const double *active_position, const double *active_charge,
                                          const double *target_positions, const double *target_charges,
                                          const double *potential_changes, int64_t n, double *displacement,
                                          int32_t *status, void *stream) {
    if (!desc || n < 0) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;
    if (!velocity || !active_position || !active_charge || !target_positions || !target_charges ||
        !potential_changes || !displacement || !status)
        return JFGPU_ERROR_ARGUMENT;
    jf::CompositeArgs a{};
    a.n = n;
    a.velocity = velocity;
    a.active_position = active_position;
    a.active_charge = active_charge;
    a.target_positions = target_positions;
    a.target_charges = target_charges;
    a.potential_changes = potential_changes;
    a.displacement = displacement;
    a.status = status;
    return jf::run(a, desc, stream, false);
}

extern "C" int jfgpu_composite_out_state(const JfgpuCompositeDesc *desc, int32_t draw_mode, const double *velocity,
                                         const double *local_positions, const double *local_charges,
                                         const int32_t *active_index, const double *target_positions,
                                         const double *target_charges, const int32_t *local_first,
                                         const double *draws, int64_t n, int32_t *new_active, double *rates,
                                         int32_t *status, void *stream) {
    if (!desc || n < 0) return JFGPU_ERROR_ARGUMENT;
    if (draw_mode != JFGPU_DRAW_VALUE && draw_mode != JFGPU_DRAW_UNIT) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;
    if (!velocity || !local_positions || !local_charges || !active_index || !target_positions || !target_charges ||
        !local_first || !draws || !new_active || !status)
        return JFGPU_ERROR_ARGUMENT;
    jf::CompositeArgs a{};
    a.draw_mode = draw_mode;
    a.n = n;
    a.velocity = velocity;
    a.local_positions = local_positions;
    a.local_charges = local_charges;
    a.active_index = active_index;
    a.target_positions = target_positions;
    a.target_charges = target_charges;
    a.local_first = local_first;
    a.draws = draws;
    a.new_active = new_active;
    a.rates = rates;
    a.status = status;
    return jf::run(a, desc, stream, true);
}

extern "C" int jfgpu_composite_bounded_out_state(const JfgpuCompositeDesc *desc, int32_t draw_mode,
                                                 const double *velocity, const double *local_positions,
                                                 const double *local_charges, const int32_t *active_index,
                                                 const double *target_positions, const double *target_charges,
                                                 const int32_t *local_first, const double *bounding_rates,
                                                 const double *draws, int64_t n, int32_t *new_active, double *rates,
                                                 int32_t *status, void *stream) {
    if (!desc || n < 0) return JFGPU_ERROR_ARGUMENT;
    if (draw_mode != JFGPU_DRAW_VALUE && draw_mode != JFGPU_DRAW_UNIT) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;
    if (!velocity || !local_positions || !local_charges || !active_index || !target_positions || !target_charges ||
        !local_first || !bounding_rates || !draws || !new_active || !status)
        return JFGPU_ERROR_ARGUMENT;
    jf::CompositeArgs a{};
    a.draw_mode = draw_mode;
    a.n = n;
    a.velocity = velocity;
    a.local_positions = local_positions;
    a.local_charges = local_charges;
    a.active_index = active_index;
    a.target_positions = target_positions;
    a.target_charges = target_charges;
    a.local_first = local_first;
    a.bounding_rates = bounding_rates;
    a.draws = draws;
    a.new_active = new_active;
    a.rates = rates;
    a.status = status;
    return jf::run(a, desc, stream, true);
}

namespace jf {

// Walker.sample_cell (walker.py:105-122): the table entry random.choice picked, then random.uniform(0.0, mean) against
// the entry's first rate (a value, or 0.0 + (mean - 0.0) * u for a unit draw u)
__global__ void walker_sample_kernel(const int32_t *first_item, const double *first_rate, const int32_t *second_item,
                                     int64_t size, double mean_rate, const int64_t *choice, const double *draws,
                                     int draw_mode, int64_t n, int32_t *items, int32_t *status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t k = choice[i];
    if (k < 0 || k >= size) {
        items[i] = -1;
        status[i] = JFGPU_STATUS_INDEX;
        return;
    }
    const double value = draw_mode == JFGPU_DRAW_UNIT ? 0.0 + (mean_rate - 0.0) * draws[i] : draws[i];
    items[i] = value <= first_rate[k] ? first_item[k] : second_item[k];
    status[i] = JFGPU_STATUS_OK;
}

}  // namespace jf

extern "C" int jfgpu_walker_sample(const int32_t *first_item, const double *first_rate, const int32_t *second_item,
                                   int64_t size, double mean_rate, const int64_t *choice, const double *draws,
                                   int32_t draw_mode, int64_t n, int32_t *items, int32_t *status, void *stream) {
    if (n < 0 || size < 0) return JFGPU_ERROR_ARGUMENT;
    if (draw_mode != JFGPU_DRAW_VALUE && draw_mode != JFGPU_DRAW_UNIT) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;
    if (!first_item || !first_rate || !second_item || !choice || !draws || !items || !status)
        return JFGPU_ERROR_ARGUMENT;
    const int threads = 128;
    const int64_t blocks = (n + threads - 1) / threads;
    jf::walker_sample_kernel<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(
        first_item, first_rate, second_item, size, mean_rate, choice, draws, draw_mode, n, items, status);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

static int launch_cell_time(jf::CellTimeArgs &a, bool veto, void *stream) {
    const int threads = 128;
    const int64_t blocks = (a.n + threads - 1) / threads;
    jf::cell_time_kernel<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(a, veto);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

extern "C" int jfgpu_composite_cell_bound_time(const double *upper, const double *lower, int64_t cells,
                                               const int32_t *relative_cell, const double *velocity,
                                               const double *active_charge, const double *target_charges,
                                               int32_t units, double dipole_charge, const double *potential_change,
                                               int64_t n, double *rate, double *time, int32_t *status,
                                               void *stream) {
    if (n < 0 || cells < 0 || units < 1 || units > jf::kMaxCompositeUnits) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;
    if (!upper || !lower || !relative_cell || !velocity || !active_charge || !target_charges || !potential_change ||
        !rate || !time || !status)
        return JFGPU_ERROR_ARGUMENT;
    jf::CellTimeArgs a{};
    a.upper = upper;
    a.lower = lower;
    a.cells = cells;
    a.n = n;
    a.relative_cell = relative_cell;
    a.velocity = velocity;
    a.active_charge = active_charge;
    a.target_charges = target_charges;
    a.units = units;
    a.dipole_charge = dipole_charge;
    a.potential_change = potential_change;
    a.rate = rate;
    a.time = time;
    a.status = status;
    return launch_cell_time(a, false, stream);
}

extern "C" int jfgpu_composite_cell_veto_time(const double *upper, const double *lower, int64_t cells,
                                              const double *walker_upper, const double *walker_lower,
                                              const int32_t *relative_cell, const double *velocity,
                                              const double *active_charge, const double *potential_change, int64_t n,
                                              double *rate, double *time, int32_t *status, void *stream) {
    if (n < 0 || cells < 0) return JFGPU_ERROR_ARGUMENT;
    if (n == 0) return JFGPU_OK;
    if (!upper || !lower || !walker_upper || !walker_lower || !relative_cell || !velocity || !active_charge ||
        !potential_change || !rate || !time || !status)
        return JFGPU_ERROR_ARGUMENT;
    jf::CellTimeArgs a{};
    a.upper = upper;
    a.lower = lower;
    a.walker_upper = walker_upper;
    a.walker_lower = walker_lower;
    a.cells = cells;
    a.n = n;
    a.relative_cell = relative_cell;
    a.velocity = velocity;
    a.active_charge = active_charge;
    a.potential_change = potential_change;
    a.rate = rate;
    a.time = time;
    a.status = status;
    return launch_cell_time(a, true, stream);
}
