// jf_engine_host.cu -- engine construction (tables) and the C ABI of the chain batch.
//
// Geometry tables follow the reference's cell system exactly:
//   exact float cell bounds .............. cuboid_cells.py:115-131 (next float up / down until int(x / side) flips)
//   relative_cell / translate ............. cuboid_periodic_cells.py:156-207 (per-axis tables)
//   nearby cells .......................... cuboid_periodic_cells.py:74-100 (distinct residues of the layer offsets)
// Far-field tables:
//   InnerPointEstimator.derivative_bound .. inner_point_estimator.py:108-163, evaluated on the GPU (estimator_kernel)
//   cell-bounding / cell-veto bounds ...... cell_bounding_potential.py:104-118, cell_veto_event_handler.py:134-159
//   Walker's alias table .................. walker.py:53-103 (built on the host in the reference's order)
//   merged-image Fourier coefficients ..... merged_image_coulomb_potential.c:77-119 (host libm, as the reference)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "jf_engine.cuh"

namespace jf {
cudaError_t launch_init(const EngineView &view, long long n_chains, const JfgpuBuffers &b, const LaunchPlan &plan);
cudaError_t launch_mirror(const EngineView &view, const JfgpuBuffers &b, long long first_chain, long long count,
                          long long first_unit, long long units, cudaStream_t stream);
cudaError_t launch_run(const EngineView &view, const JfgpuBuffers &b, long long first, long long count,
                       long long max_events, double stop_q, double stop_r, int mode, JfgpuEvent *log,
                       long long log_capacity, int uniform_potential, int uniform_far, void *lists, void *refined,
                       void *queue, void *ahead, void *settle, long long n_chains, const LaunchPlan &plan,
                       long long *launches);
size_t refine_list_bytes();
size_t far_ahead_bytes();
size_t refined_bytes();
size_t refine_queue_bytes(long long n_chains);
void *graph_cache_create();
void graph_cache_destroy(void *cache);
cudaError_t launch_observe(const EngineView &view, long long first, long long count, int max_n,
                           const float4 *positions32, int bins, double r_max, double *energy,
                           unsigned long long *histogram, const LaunchPlan &plan);
}  // namespace jf

using namespace jf;

// CUDA events around the launches: one event before the first launch on a stream, one after every launch, so
// that a launch's time is the interval between its stream's previous event and its own
class EventClock : public KernelClock {
  public:
    ~EventClock() override {
        for (cudaEvent_t ev : pool_) cudaEventDestroy(ev);
    }
    void begin(cudaStream_t stream) override {
        int i = next();
        if (i < 0) return;
        cudaEventRecord(pool_[i], stream);
        last_[stream] = i;
    }
    void end(cudaStream_t stream, int kind) override {
        auto it = last_.find(stream);
        int i = next();
        if (i < 0 || it == last_.end()) return;
        cudaEventRecord(pool_[i], stream);
        marks_.push_back({kind, it->second, i});
        it->second = i;
    }
    // waits for the recorded events and adds their intervals to the totals
    int collect() {
        int error = JFGPU_OK;
        for (const Mark &m : marks_) {
            float ms = 0.0f;
            if (cudaEventSynchronize(pool_[m.after]) != cudaSuccess ||
                cudaEventElapsedTime(&ms, pool_[m.before], pool_[m.after]) != cudaSuccess) {
                error = JFGPU_ERROR_CUDA;
                continue;
            }
            milliseconds[m.kind] += ms;
            launches[m.kind] += 1;
        }
        marks_.clear();
        last_.clear();
        used_ = 0;
        return failed_ ? JFGPU_ERROR_CUDA : error;
    }
    double milliseconds[JFGPU_KERNEL_KINDS] = {};
    int64_t launches[JFGPU_KERNEL_KINDS] = {};

  private:
    struct Mark {
        int kind, before, after;
    };
    int next() {
        if (used_ == pool_.size()) {
            cudaEvent_t ev;
            if (cudaEventCreate(&ev) != cudaSuccess) {
                failed_ = true;
                return -1;
            }
            pool_.push_back(ev);
        }
        return (int)used_++;
    }
    std::vector<cudaEvent_t> pool_;
    size_t used_ = 0;
    bool failed_ = false;
    std::map<cudaStream_t, int> last_;
    std::vector<Mark> marks_;
};

struct JfgpuEngine {
    std::vector<JfgpuChainDesc> descs;
    std::vector<ChainDev> chains;
    std::vector<SpeciesDev> species;
    std::vector<std::vector<double>> species_upper, species_lower;  // host copies of the bound tables
    std::vector<int> chain_species;
    std::vector<void *> allocations;
    EngineView view{};
    int64_t particles = 0, occupancy_slots = 0, table_bytes = 0;
    int64_t launches = 0;
    int block_warps = 4;
    int refine_limit = JFGPU_REFINE_LIST_MAX;
    void *refine_lists = nullptr;  // per-chain refine lists of the mixed-precision rounds
    void *refined = nullptr;       // per-chain FP64 re-solves of the first list entries
    void *refine_queue = nullptr;  // the re-solves queued by screening path
    void *far_ahead = nullptr;     // per chain: the far units' smallest keyed draws of its next event
    void *settle = nullptr;        // per chain: inputs of its settle that have arrived in the running round
    int groups = 1;                // chain groups of the mixed mode, each on a stream of its own
    cudaStream_t group_streams[8] = {};
    cudaEvent_t fork = nullptr, join[8] = {};
    EventClock *clock = nullptr;   // per-kernel timing, null while off
    void *graphs = nullptr;        // captured round segments of the mixed mode (null: plain launches)
};

namespace {

double py_sum(const std::vector<double> &values) {  // builtin sum() of CPython 3.12 (Neumaier)
    if (values.empty()) return 0.0;
    double f = 0.0 + values[0];
    double c = 0.0;
    for (size_t i = 1; i < values.size(); ++i) {
        double x = values[i];
        double t = f + x;
        if (std::fabs(f) >= std::fabs(x))
            c += (f - t) + x;
        else
            c += (x - t) + f;
        f = t;
    }
    if (c != 0.0 && std::isfinite(c)) f += c;
    return f;
}

double next_up(double x) {
    if (std::isnan(x) || (std::isinf(x) && x > 0)) return x;
    if (x == 0.0) x = 0.0;
    return std::nextafter(x, INFINITY);
}

double next_down(double x) { return -next_up(-x); }

}  // namespace

namespace jf {

void cell_bounds(double length, int m, std::vector<double> &lo, std::vector<double> &hi) {
    double side = length / m;
    lo.resize(m);
    hi.resize(m);
    for (int i = 0; i < m; ++i) {
        double lower = i * side;
        double upper = (i + 1) * side;
        if (lower > 0.0) {
            while ((long long)(lower / side) == i) lower = next_down(lower);
            while ((long long)(lower / side) < i) lower = next_up(lower);
        }
        while ((long long)(upper / side) == i) upper = next_up(upper);
        while ((long long)(upper / side) > i) upper = next_down(upper);
        lo[i] = lower;
        hi[i] = upper;
    }
}

int walker_build(const std::vector<int> &items, const std::vector<double> &rates, HostWalker &w) {
    struct Item {
        int item;
        double rate;
    };
    int n = (int)items.size();
    if (n == 0) return JFGPU_ERROR_TABLE;
    w.total_rate = py_sum(rates);
    w.mean_rate = w.total_rate / n;
    std::vector<Item> small, large;
    for (int i = 0; i < n; ++i) {
        if (!(rates[i] >= 0.0)) return JFGPU_ERROR_TABLE;
        Item it{items[i], rates[i]};
        if (rates[i] > w.mean_rate)
            large.push_back(it);
        else
            small.push_back(it);
    }
    while (!small.empty() && !large.empty()) {
        Item s = small.back();
        small.pop_back();
        Item l = large.back();
        large.pop_back();
        w.first_item.push_back(s.item);
        w.first_rate.push_back(s.rate);
        w.second_item.push_back(l.item);
        l.rate -= w.mean_rate - s.rate;
        if (l.rate < w.mean_rate)
            small.push_back(l);
        else
            large.push_back(l);
    }
    for (auto *list : {&small, &large}) {
        while (!list->empty()) {
            Item s = list->back();
            list->pop_back();
            double ratio = s.rate / w.mean_rate;
            if (!(1 - 1e-6 < ratio && ratio < 1 + 1e-6)) return JFGPU_ERROR_TABLE;
            w.first_item.push_back(s.item);
            w.first_rate.push_back(w.mean_rate);
            w.second_item.push_back(-1);
        }
    }
    return JFGPU_OK;
}

}  // namespace jf

namespace {

template <typename T>
T *device_copy(JfgpuEngine *e, const std::vector<T> &host, cudaStream_t stream, int &error) {
    if (host.empty()) return nullptr;
    void *ptr = nullptr;
    size_t bytes = sizeof(T) * host.size();
    if (cudaMalloc(&ptr, bytes) != cudaSuccess) {
        error = JFGPU_ERROR_ALLOCATION;
        return nullptr;
    }
    e->allocations.push_back(ptr);
    e->table_bytes += (int64_t)bytes;
    if (cudaMemcpyAsync(ptr, host.data(), bytes, cudaMemcpyHostToDevice, stream) != cudaSuccess)
        error = JFGPU_ERROR_CUDA;
    return static_cast<T *>(ptr);
}


}  // namespace

namespace jf {

// LennardJonesPotential.__init__ (lennard_jones_potential.py:43-61)
MH make_lj(double prefactor, double sigma) {
    MH h;
    memset(&h, 0, sizeof(h));
    h.kind = 0;
    h.prefactor = prefactor;
    h.sigma = sigma;
    h.r0 = sigma * std::pow(2.0, 1.0 / 6.0);  // characteristic_length * 2 ** (1 / 6)
    h.r0_squared = std::pow(h.r0, 2.0);       // equilibrium_separation ** 2
    h.six = ip_make(6.0, -prefactor * std::pow(sigma, 6.0));
    h.twelve = ip_make(12.0, prefactor * std::pow(sigma, 12.0));
    return h;
}

// DisplacedEvenPowerPotential.__init__ (displaced_even_power_potential.py:44-71)
MH make_displaced(double r0, int power, double prefactor) {
    MH h;
    memset(&h, 0, sizeof(h));
    h.kind = 1;
    h.prefactor = prefactor;
    h.r0 = r0;
    h.r0_squared = r0 * r0;  // displaced_even_power_potential.py:68
    h.power = (double)power;
    h.inverse_power = 1.0 / (double)power;
    return h;
}

// merged_image_coulomb_potential.c:77-119
std::vector<double> fourier_table(int fc, double alpha, double length) {
    int n = fc + 1;
    std::vector<double> t((size_t)n * n * n, 0.0);
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++)
            for (int i = 1; i < n; i++) {
                double coefficient = (j == 0 && k == 0) ? 1.0 : ((k == 0 || j == 0) ? 2.0 : 4.0);
                double norm_sq = i * i + j * j + k * k;
                t[(i * n + j) * n + k] = 4.0 * i * coefficient / (norm_sq * length * length) *
                                         std::exp(-M_PI * M_PI * norm_sq / (alpha * alpha));
            }
    return t;
}

// the terms of the merged-image sum in the order of merged_image_coulomb_potential.c:205-274: real-space images
// (i, j, k) with i^2 + j^2 + k^2 <= position_cutoff^2, Fourier rows (i, j, last k) with i >= 1
void merged_image_terms(int fc, int pc, std::vector<int4> &images, std::vector<int4> &rows) {
    for (int k = -pc; k < pc + 1; k++) {
        int cutoff_y = (int)std::sqrt((double)(pc * pc - k * k));
        for (int j = -cutoff_y; j < cutoff_y + 1; j++) {
            int cutoff_x = (int)std::sqrt((double)(pc * pc - j * j - k * k));
            for (int i = -cutoff_x; i < cutoff_x + 1; i++) images.push_back(make_int4(i, j, k, 0));
        }
    }
    for (int i = 1; i < fc + 1; i++) {
        int cutoff_y = (int)std::sqrt((double)(fc * fc - i * i));
        for (int j = 0; j < cutoff_y + 1; j++) {
            int cutoff_x = (int)std::sqrt((double)(fc * fc - i * i - j * j));
            rows.push_back(make_int4(i, j, cutoff_x, 0));
        }
    }
}

MIC make_mic(int fc, int pc, double alpha, double length, const double *fourier) {
    MIC m;
    m.fourier_cutoff = fc;
    m.fourier_cutoff_sq = fc * fc;
    m.position_cutoff = pc;
    m.position_cutoff_sq = pc * pc;
    m.alpha_over_length = alpha / length;
    m.alpha_over_length_sq = alpha * alpha / (length * length);
    m.two_alpha_over_length_root_pi = 2.0 * alpha / (length * std::sqrt(M_PI));
    m.system_length = length;
    m.two_pi_over_length = 2.0 * M_PI / length;
    m.fourier = fourier;
    return m;
}

}  // namespace jf

// ---------------------------------------------------------------------------------------------------------------
// estimator scan: one block per (far cell, direction); the grid points of InnerPointEstimator.derivative_bound
// ---------------------------------------------------------------------------------------------------------------
namespace jf {

struct EstimatorArgs {
    MH lj;
    MIC mic;
    int potential;
    int points;
    double half, length, coulomb_prefactor;
    const int32_t *cells;    // far cells
    const double *lower;     // [cells][3]
    const double *upper;     // [cells][3]
    double *max_out;         // [cells][3]
    double *min_out;         // [cells][3]
    int32_t *status;
};

__global__ void estimator_kernel(EstimatorArgs a) {
    const int index = blockIdx.x;  // far cell
    const int direction = blockIdx.y;
    const int pps = a.points;
    const int total = (pps + 1) * (pps + 1) * (pps + 1);
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = a.lower[index * 3 + k];
        hi[k] = a.upper[index * 3 + k];
    }
    double vmax = -kInf, vmin = kInf;
    int status = 0;
    for (int p = threadIdx.x; p < total; p += blockDim.x) {
        int iz = p % (pps + 1), iy = (p / (pps + 1)) % (pps + 1), ix = p / ((pps + 1) * (pps + 1));
        double s[3];
        s[0] = lo[0] + ((hi[0] - lo[0]) * ix) / pps;
        s[1] = lo[1] + ((hi[1] - lo[1]) * iy) / pps;
        s[2] = lo[2] + ((hi[2] - lo[2]) * iz) / pps;
        for (int k = 0; k < 3; ++k) s[k] = py_mod(s[k] + a.half, a.length) - a.half;
        double derivative;
        if (a.potential == JFGPU_POT_LENNARD_JONES) {
            int st = mh_std_derivative(a.lj, direction, s, derivative);
            if (st) {
                status = st;
                continue;
            }
            derivative = derivative * 1.0;
        } else {
            derivative = mic_std_derivative(a.mic, a.coulomb_prefactor, direction, s, 1.0, 1.0) * 1.0;
        }
        if (derivative > vmax) vmax = derivative;
        if (derivative < vmin) vmin = derivative;
    }
    __shared__ double smax[256], smin[256];
    __shared__ int sst[256];
    smax[threadIdx.x] = vmax;
    smin[threadIdx.x] = vmin;
    sst[threadIdx.x] = status;
    __syncthreads();
    for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride) {
            if (smax[threadIdx.x + stride] > smax[threadIdx.x]) smax[threadIdx.x] = smax[threadIdx.x + stride];
            if (smin[threadIdx.x + stride] < smin[threadIdx.x]) smin[threadIdx.x] = smin[threadIdx.x + stride];
            sst[threadIdx.x] = max(sst[threadIdx.x], sst[threadIdx.x + stride]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.max_out[index * 3 + direction] = smax[0];
        a.min_out[index * 3 + direction] = smin[0];
        if (sst[0]) atomicMax(a.status, sst[0]);
    }
}

}  // namespace jf

namespace {

struct SpeciesKey {
    int potential, far, m, layers, fc, pc, points;
    double length, lj_prefactor, lj_sigma, coulomb_prefactor, alpha, estimator_prefactor;
    bool operator<(const SpeciesKey &o) const {
        return std::tie(potential, far, m, layers, fc, pc, points, length, lj_prefactor, lj_sigma, coulomb_prefactor,
                        alpha, estimator_prefactor) <
               std::tie(o.potential, o.far, o.m, o.layers, o.fc, o.pc, o.points, o.length, o.lj_prefactor, o.lj_sigma,
                        o.coulomb_prefactor, o.alpha, o.estimator_prefactor);
    }
};

int build_species(JfgpuEngine *e, const JfgpuChainDesc &d, const std::vector<double> &cmin,
                  const std::vector<double> &cmax, const std::vector<unsigned char> &near_axis, cudaStream_t stream,
                  SpeciesDev &sp, std::vector<double> &upper_host, std::vector<double> &lower_host) {
    memset(&sp, 0, sizeof(sp));
    int error = JFGPU_OK;
    const int m = d.cells_per_side;
    const int ncells = m * m * m;
    if (d.potential == JFGPU_POT_LENNARD_JONES) {
        sp.lj = make_lj(d.lj_prefactor, d.lj_sigma);
        sp.lj32[0] = (float)sp.lj.twelve.prefactor;
        sp.lj32[1] = (float)sp.lj.six.prefactor;
        sp.lj32[2] = (float)(4.0 / sp.lj.prefactor);
        sp.lj32[3] = (float)(sp.lj.sigma * sp.lj.sigma);
        sp.lj32[4] = (float)sp.lj.r0_squared;
    }
    if (d.potential == JFGPU_POT_COULOMB) {
        std::vector<double> table = fourier_table(d.fourier_cutoff, d.ewald_alpha, d.system_length);
        const double *dev = device_copy(e, table, stream, error);
        if (error) return error;
        sp.mic = make_mic(d.fourier_cutoff, d.position_cutoff, d.ewald_alpha, d.system_length, dev);
        // the terms of the sum as lists, for the warp-shared evaluation of the thinning derivative
        std::vector<int4> images, rows;
        merged_image_terms(d.fourier_cutoff, d.position_cutoff, images, rows);
        std::vector<int4> terms(images);
        terms.insert(terms.end(), rows.begin(), rows.end());
        const int4 *dev_terms = device_copy(e, terms, stream, error);
        if (error) return error;
        sp.mic_terms = dev_terms;
        sp.mic_images = (int)images.size();
        sp.mic_rows = (int)rows.size();
        std::vector<float> table32(table.begin(), table.end());
        sp.mic_fourier32 = device_copy(e, table32, stream, error);
        if (error) return error;
    }
    if (d.far == JFGPU_FAR_NONE) return JFGPU_OK;
    if (d.max_occupants != 1) return JFGPU_ERROR_ARGUMENT;
    // far cells: not nearby the zero cell, in cell order (cell_bounding_potential.py:104-118)
    std::vector<int32_t> far_cells;
    std::vector<double> lower, upper;
    for (int cell = 0; cell < ncells; ++cell) {
        int a[3] = {cell % m, (cell / m) % m, cell / (m * m)};
        if (near_axis[a[0]] && near_axis[a[1]] && near_axis[a[2]]) continue;
        far_cells.push_back(cell);
        for (int k = 0; k < 3; ++k) {
            lower.push_back(cmin[a[k]] - cmax[0]);
            upper.push_back(cmax[a[k]] - cmin[0]);
        }
    }
    int nfar = (int)far_cells.size();
    if (nfar == 0) return JFGPU_ERROR_TABLE;
    std::vector<double> zeros((size_t)nfar * 3, 0.0);
    double *d_lower = device_copy(e, lower, stream, error);
    double *d_upper = device_copy(e, upper, stream, error);
    double *d_max = device_copy(e, zeros, stream, error);
    double *d_min = device_copy(e, zeros, stream, error);
    int32_t *d_status = device_copy(e, std::vector<int32_t>{0}, stream, error);
    if (error) return error;
    EstimatorArgs args;
    args.lj = sp.lj;
    args.mic = sp.mic;
    args.potential = d.potential;
    args.points = d.estimator_points;
    args.half = d.system_length / 2.0;
    args.length = d.system_length;
    args.coulomb_prefactor = d.coulomb_prefactor;
    args.cells = nullptr;
    args.lower = d_lower;
    args.upper = d_upper;
    args.max_out = d_max;
    args.min_out = d_min;
    args.status = d_status;
    estimator_kernel<<<dim3((unsigned)nfar, 3), 256, 0, stream>>>(args);
    e->launches += 1;
    if (cudaGetLastError() != cudaSuccess) return JFGPU_ERROR_CUDA;
    std::vector<double> vmax((size_t)nfar * 3), vmin((size_t)nfar * 3);
    int32_t st = 0;
    if (cudaMemcpyAsync(vmax.data(), d_max, sizeof(double) * vmax.size(), cudaMemcpyDeviceToHost, stream) ||
        cudaMemcpyAsync(vmin.data(), d_min, sizeof(double) * vmin.size(), cudaMemcpyDeviceToHost, stream) ||
        cudaMemcpyAsync(&st, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, stream) ||
        cudaStreamSynchronize(stream))
        return JFGPU_ERROR_CUDA;
    if (st) return JFGPU_ERROR_TABLE;
    // prefactor (inner_point_estimator.py:154-163), empirical bound infinite
    upper_host.assign((size_t)ncells * 3, 0.0);
    lower_host.assign((size_t)ncells * 3, 0.0);
    const double pref = d.estimator_prefactor;
    for (int i = 0; i < nfar; ++i)
        for (int k = 0; k < 3; ++k) {
            double ub = vmax[i * 3 + k], lb = vmin[i * 3 + k];
            ub = ub > 0.0 ? ub * pref : ub / pref;
            lb = lb > 0.0 ? lb / pref : lb * pref;
            upper_host[far_cells[i] * 3 + k] = ub;
            lower_host[far_cells[i] * 3 + k] = -lb;
        }
    sp.bound_upper = device_copy(e, upper_host, stream, error);
    sp.bound_lower = device_copy(e, lower_host, stream, error);
    std::vector<float> upper32(upper_host.begin(), upper_host.end());
    sp.bound_upper32 = device_copy(e, upper32, stream, error);
    // the largest FP32 rate of each direction over the far cells (nearby cells hold 0): a keyed draw above
    // reject * this bound rejects its unit without reading where the unit is
    for (int k = 0; k < 3; ++k) {
        float largest = 0.0f;
        for (int cell = 0; cell < ncells; ++cell)
            if (upper32[cell * 3 + k] > largest) largest = upper32[cell * 3 + k];
        sp.far_rate_max32[k] = largest;
    }
    if (error) return error;
    if (d.far == JFGPU_FAR_CELL_VETO) {
        for (int which = 0; which < 2; ++which)
            for (int k = 0; k < 3; ++k) {
                std::vector<int> items;
                std::vector<double> rates;
                for (int cell : far_cells) {
                    double r = which == 0 ? upper_host[cell * 3 + k] : lower_host[cell * 3 + k];
                    items.push_back(cell);
                    rates.push_back(r > 0.0 ? r : 0.0);
                }
                HostWalker hw;
                int werr = walker_build(items, rates, hw);
                if (werr) return werr;
                WalkerDev &wd = sp.walker[which][k];
                wd.first_item = device_copy(e, hw.first_item, stream, error);
                wd.second_item = device_copy(e, hw.second_item, stream, error);
                wd.first_rate = device_copy(e, hw.first_rate, stream, error);
                wd.size = (int32_t)hw.first_item.size();
                wd.total_rate = hw.total_rate;
                wd.mean_rate = hw.mean_rate;
                if (error) return error;
            }
    }
    return JFGPU_OK;
}

}  // namespace

// Walker's alias table over n items in the order given (walker.py:53-103), built on the host as the engine builds
// its cell-veto tables: first_item / first_rate / second_item [n] (second_item -1 for an entry of one item), the
// total rate (builtin sum) and the mean rate.  JFGPU_ERROR_TABLE for a negative rate or a leftover entry whose rate
// strays from the mean by 1e-6 or more (the reference's assertions).
extern "C" int jfgpu_walker_table(const int32_t *items, const double *rates, int64_t n, int32_t *first_item,
                                  double *first_rate, int32_t *second_item, double *total_rate, double *mean_rate) {
    if (n < 1 || n > INT32_MAX || !items || !rates || !first_item || !first_rate || !second_item || !total_rate ||
        !mean_rate)
        return JFGPU_ERROR_ARGUMENT;
    std::vector<int> item_list(items, items + n);
    std::vector<double> rate_list(rates, rates + n);
    HostWalker w;
    const int error = walker_build(item_list, rate_list, w);
    if (error) return error;
    for (int64_t k = 0; k < n; ++k) {
        first_item[k] = w.first_item[k];
        first_rate[k] = w.first_rate[k];
        second_item[k] = w.second_item[k];
    }
    *total_rate = w.total_rate;
    *mean_rate = w.mean_rate;
    return JFGPU_OK;
}

extern "C" {

int jfgpu_version(void) { return 1; }

const char *jfgpu_error_string(int code) {
    switch (code) {
    case JFGPU_OK:
        return "ok";
    case JFGPU_ERROR_CUDA:
        return "CUDA runtime error";
    case JFGPU_ERROR_ARGUMENT:
        return "invalid argument";
    case JFGPU_ERROR_ALLOCATION:
        return "device allocation failed";
    case JFGPU_ERROR_TABLE:
        return "table construction failed (estimator or Walker table)";
    default:
        return "unknown error";
    }
}

void jfgpu_engine_destroy(JfgpuEngine *engine) {
    if (!engine) return;
    for (int g = 0; g < 8; ++g) {
        if (engine->group_streams[g]) cudaStreamDestroy(engine->group_streams[g]);
        if (engine->join[g]) cudaEventDestroy(engine->join[g]);
    }
    if (engine->fork) cudaEventDestroy(engine->fork);
    delete engine->clock;
    graph_cache_destroy(engine->graphs);
    for (void *p : engine->allocations) cudaFree(p);
    delete engine;
}

int jfgpu_engine_create(const JfgpuChainDesc *chains, int64_t n_chains, void *stream_ptr, JfgpuEngine **out) {
    if (!chains || n_chains <= 0 || !out) return JFGPU_ERROR_ARGUMENT;
    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    JfgpuEngine *e = new JfgpuEngine();
    e->descs.assign(chains, chains + n_chains);
    std::vector<double> cmin_pool, cmax_pool;
    std::vector<int16_t> rel_pool, tra_pool;
    std::map<std::pair<double, int>, std::pair<int, int>> geometry;  // (L, m) -> (geom offset, table offset)
    std::map<std::pair<double, int>, int> geometry_mod;                // (L, m) -> tables are modular arithmetic
    std::map<SpeciesKey, int> species_index;
    int error = JFGPU_OK;
    for (int64_t c = 0; c < n_chains && !error; ++c) {
        const JfgpuChainDesc &d = chains[c];
        const int m = d.cells_per_side;
        if (d.n < 2 || d.n > (1 << 20) || m < 1 || m > kMaxResidues || d.neighbor_layers < 0 ||
            d.neighbor_layers > 7 || d.max_occupants < 1 || !(d.system_length > 0.0) || d.initial_active < 0 ||
            d.initial_active >= d.n || d.initial_direction < 0 || d.initial_direction > 2 || !(d.speed > 0.0) ||
            !(d.beta > 0.0) || !(d.chain_time > 0.0) || d.potential < 0 || d.potential > 2 || d.far < 0 ||
            d.far > 2 || (d.potential == JFGPU_POT_HARD_SPHERE && d.far != JFGPU_FAR_NONE) ||
            (d.far != JFGPU_FAR_NONE && d.estimator_points < 1)) {
            error = JFGPU_ERROR_ARGUMENT;
            break;
        }
        std::vector<double> lo, hi;
        cell_bounds(d.system_length, m, lo, hi);
        auto gkey = std::make_pair(d.system_length, m);
        if (!geometry.count(gkey)) {
            int goff = (int)cmin_pool.size();
            int toff = (int)rel_pool.size();
            cmin_pool.insert(cmin_pool.end(), lo.begin(), lo.end());
            cmax_pool.insert(cmax_pool.end(), hi.begin(), hi.end());
            double side = d.system_length / m;
            for (int a = 0; a < m; ++a)
                for (int b = 0; b < m; ++b) {
                    double center = (hi[a] + lo[a]) / 2.0;
                    rel_pool.push_back((int16_t)(long long)(py_mod(center - lo[b], d.system_length) / side));
                    tra_pool.push_back((int16_t)(long long)(py_mod(center + lo[b], d.system_length) / side));
                }
            int is_mod = 1;
            for (int a = 0; a < m; ++a)
                for (int b = 0; b < m; ++b) {
                    if (rel_pool[toff + a * m + b] != ((a - b) % m + m) % m) is_mod = 0;
                    if (tra_pool[toff + a * m + b] != (a + b) % m) is_mod = 0;
                }
            geometry[gkey] = std::make_pair(goff, toff);
            geometry_mod[gkey] = is_mod;
        }
        std::vector<unsigned char> near_axis(m, 0);
        for (int o = -d.neighbor_layers; o <= d.neighbor_layers; ++o) near_axis[((o % m) + m) % m] = 1;
        ChainDev ch;
        memset(&ch, 0, sizeof(ch));
        ch.potential = d.potential;
        ch.far = d.far;
        ch.n = d.n;
        ch.m = m;
        ch.ncells = m * m * m;
        ch.max_occ = d.max_occupants;
        ch.initial_active = d.initial_active;
        ch.initial_direction = d.initial_direction;
        ch.geom_offset = geometry[gkey].first;
        ch.table_offset = geometry[gkey].second;
        ch.rel_is_mod = geometry_mod[gkey];
        ch.n_res = 0;
        ch.near_mask = 0;
        for (int r = 0; r < m; ++r)
            if (near_axis[r]) {
                ch.res[ch.n_res++] = r;
                ch.near_mask |= 1ull << r;
            }
        ch.pos_off = e->particles;
        ch.occ_off = e->occupancy_slots;
        e->particles += d.n;
        e->occupancy_slots += (int64_t)ch.ncells * d.max_occupants;
        ch.L = d.system_length;
        ch.half = d.system_length / 2.0;
        ch.side = d.system_length / m;
        ch.inv_side = 1.0 / ch.side;
        ch.beta = d.beta;
        ch.chain_time = d.chain_time;
        ch.speed = d.speed;
        ch.diameter_sq = d.hs_radius > 0.0 ? 4.0 * d.hs_radius * d.hs_radius : 0.0;
        ch.bound_prefactor = d.bound_prefactor;
        ch.coulomb_prefactor = d.coulomb_prefactor;
        ch.L32 = (float)d.system_length;
        ch.half32 = (float)(d.system_length / 2.0);
        ch.ulp_margin32 = (float)(16.0 * d.system_length / 16777216.0);
        ch.screen_abs32 = (float)(d.system_length / 65536.0);
        ch.speed32 = (float)d.speed;
        ch.inv_beta32 = (float)(1.0 / d.beta);
        ch.diameter_sq32 = (float)ch.diameter_sq;
        ch.key = d.rng_key;
        SpeciesKey key{d.potential, d.far, m, d.neighbor_layers, d.fourier_cutoff, d.position_cutoff,
                       d.estimator_points, d.system_length, d.lj_prefactor, d.lj_sigma, d.coulomb_prefactor,
                       d.ewald_alpha, d.estimator_prefactor};
        auto it = species_index.find(key);
        if (it == species_index.end()) {
            SpeciesDev sp;
            std::vector<double> up, low;
            error = build_species(e, d, lo, hi, near_axis, stream, sp, up, low);
            if (error) break;
            int index = (int)e->species.size();
            e->species.push_back(sp);
            e->species_upper.push_back(up);
            e->species_lower.push_back(low);
            it = species_index.emplace(key, index).first;
        }
        ch.species = it->second;
        e->chain_species.push_back(it->second);
        e->chains.push_back(ch);
    }
    if (!error) {
        e->view.chains = device_copy(e, e->chains, stream, error);
        e->view.species = device_copy(e, e->species, stream, error);
        e->view.cell_min = device_copy(e, cmin_pool, stream, error);
        e->view.cell_max = device_copy(e, cmax_pool, stream, error);
        e->view.rel = device_copy(e, rel_pool, stream, error);
        e->view.tra = device_copy(e, tra_pool, stream, error);
        std::vector<unsigned char> lists(refine_list_bytes() * (size_t)n_chains, 0);
        e->refine_lists = device_copy(e, lists, stream, error);
        std::vector<unsigned char> slots(refined_bytes() * (size_t)n_chains, 0);
        e->refined = device_copy(e, slots, stream, error);
        std::vector<unsigned char> queue(refine_queue_bytes(n_chains), 0);
        e->refine_queue = device_copy(e, queue, stream, error);
        std::vector<unsigned char> ahead(far_ahead_bytes() * (size_t)n_chains, 0);  // zero: no listed event
        e->far_ahead = device_copy(e, ahead, stream, error);
        std::vector<int32_t> settle((size_t)n_chains, 0);
        e->settle = device_copy(e, settle, stream, error);
        if (!error && cudaStreamSynchronize(stream) != cudaSuccess) error = JFGPU_ERROR_CUDA;
    }
    if (error) {
        jfgpu_engine_destroy(e);
        return error;
    }
    e->graphs = graph_cache_create();
    *out = e;
    return JFGPU_OK;
}

int jfgpu_engine_layout(const JfgpuEngine *e, JfgpuLayout *layout) {
    if (!e || !layout) return JFGPU_ERROR_ARGUMENT;
    layout->n_chains = (int64_t)e->chains.size();
    layout->particles = e->particles;
    layout->occupancy_slots = e->occupancy_slots;
    layout->table_bytes = e->table_bytes;
    return JFGPU_OK;
}

int jfgpu_engine_offsets(const JfgpuEngine *e, int64_t *particle_offset, int64_t *occupancy_offset) {
    if (!e) return JFGPU_ERROR_ARGUMENT;
    for (size_t c = 0; c < e->chains.size(); ++c) {
        if (particle_offset) particle_offset[c] = e->chains[c].pos_off;
        if (occupancy_offset) occupancy_offset[c] = e->chains[c].occ_off;
    }
    return JFGPU_OK;
}

int jfgpu_engine_bounds(const JfgpuEngine *e, int64_t chain, double *upper, double *lower, int64_t capacity) {
    if (!e || chain < 0 || chain >= (int64_t)e->chains.size()) return JFGPU_ERROR_ARGUMENT;
    const std::vector<double> &up = e->species_upper[e->chain_species[chain]];
    const std::vector<double> &low = e->species_lower[e->chain_species[chain]];
    if ((int64_t)up.size() > capacity) return JFGPU_ERROR_ARGUMENT;
    if (upper) memcpy(upper, up.data(), sizeof(double) * up.size());
    if (lower) memcpy(lower, low.data(), sizeof(double) * low.size());
    return JFGPU_OK;
}

int64_t jfgpu_engine_launch_count(const JfgpuEngine *e) { return e ? e->launches : -1; }

int jfgpu_chains_set_block_warps(JfgpuEngine *e, int32_t warps) {
    if (!e || warps < 1 || warps > 8) return JFGPU_ERROR_ARGUMENT;
    e->block_warps = warps;
    return JFGPU_OK;
}

int jfgpu_chains_set_refine_limit(JfgpuEngine *e, int32_t limit) {
    if (!e || limit < 1 || limit > JFGPU_REFINE_LIST_MAX) return JFGPU_ERROR_ARGUMENT;
    e->refine_limit = limit;
    return JFGPU_OK;
}

static bool buffers_ok(const JfgpuEngine *e, const JfgpuBuffers *b) {
    return e && b && b->positions && b->positions32 && b->occupancy && b->surplus && b->roles && b->state &&
           b->cell_slots;
}

int jfgpu_chains_set_groups(JfgpuEngine *e, int32_t groups) {
    if (!e || groups < 1 || groups > 8) return JFGPU_ERROR_ARGUMENT;
    // the streams and events are made once, on the engine's device, the first time more than one group is asked for
    for (int g = 0; g < groups && groups > 1; ++g) {
        if (!e->group_streams[g] && cudaStreamCreateWithFlags(&e->group_streams[g], cudaStreamNonBlocking) != cudaSuccess)
            return JFGPU_ERROR_CUDA;
        if (!e->join[g] && cudaEventCreateWithFlags(&e->join[g], cudaEventDisableTiming) != cudaSuccess)
            return JFGPU_ERROR_CUDA;
    }
    if (groups > 1 && !e->fork && cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess)
        return JFGPU_ERROR_CUDA;
    e->groups = groups;
    return JFGPU_OK;
}

int jfgpu_chains_refresh_mirror(JfgpuEngine *e, const JfgpuBuffers *b, int64_t first, int64_t count,
                                void *stream_ptr) {
    if (!e || !b || !b->positions || !b->positions32 || !b->occupancy || !b->cell_slots || first < 0 || count < 0 ||
        first + count > (int64_t)e->chains.size())
        return JFGPU_ERROR_ARGUMENT;
    if (count == 0) return JFGPU_OK;
    const long long first_unit = e->chains[first].pos_off;
    const long long last_unit = e->chains[first + count - 1].pos_off + e->chains[first + count - 1].n;
    cudaError_t err = launch_mirror(e->view, *b, first, count, first_unit, last_unit - first_unit,
                                    static_cast<cudaStream_t>(stream_ptr));
    e->launches += 2;
    return err == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

int jfgpu_chains_set_graphs(JfgpuEngine *e, int32_t enable) {
    if (!e) return JFGPU_ERROR_ARGUMENT;
    if (enable && !e->graphs) e->graphs = graph_cache_create();
    if (!enable && e->graphs) {
        graph_cache_destroy(e->graphs);
        e->graphs = nullptr;
    }
    return JFGPU_OK;
}

int jfgpu_engine_set_timing(JfgpuEngine *e, int32_t enable) {
    if (!e || enable < 0) return JFGPU_ERROR_ARGUMENT;
    if (enable && !e->clock) e->clock = new EventClock();
    if (enable) e->clock->stride = enable;
    if (!enable && e->clock) {
        e->clock->collect();
        delete e->clock;
        e->clock = nullptr;
    }
    return JFGPU_OK;
}

int jfgpu_engine_kernel_times(JfgpuEngine *e, double *milliseconds, int64_t *launches, int32_t reset) {
    if (!e) return JFGPU_ERROR_ARGUMENT;
    int error = JFGPU_OK;
    for (int k = 0; k < JFGPU_KERNEL_KINDS; ++k) {
        if (milliseconds) milliseconds[k] = 0.0;
        if (launches) launches[k] = 0;
    }
    if (!e->clock) return JFGPU_OK;
    error = e->clock->collect();
    for (int k = 0; k < JFGPU_KERNEL_KINDS; ++k) {
        if (milliseconds) milliseconds[k] = e->clock->milliseconds[k];
        if (launches) launches[k] = e->clock->launches[k];
        if (reset) {
            e->clock->milliseconds[k] = 0.0;
            e->clock->launches[k] = 0;
        }
    }
    return error;
}

static LaunchPlan make_plan(const JfgpuEngine *e, void *stream_ptr);

int jfgpu_chains_observe(JfgpuEngine *e, const JfgpuBuffers *b, int64_t first, int64_t count, int32_t bins,
                         double r_max, double *energy, uint64_t *histogram, void *stream_ptr) {
    if (!e || !b || !b->positions32 || first < 0 || count < 0 || first + count > (int64_t)e->chains.size() ||
        (histogram && (bins < 1 || bins > 4096 || !(r_max > 0.0))))
        return JFGPU_ERROR_ARGUMENT;
    if (count == 0 || (!energy && !histogram)) return JFGPU_OK;
    int max_n = 0;
    for (int64_t c = first; c < first + count; ++c) max_n = e->chains[c].n > max_n ? e->chains[c].n : max_n;
    if (!histogram) bins = 1;
    cudaError_t err = launch_observe(e->view, first, count, max_n, reinterpret_cast<const float4 *>(b->positions32),
                                     bins, histogram ? r_max : 1.0, energy,
                                     reinterpret_cast<unsigned long long *>(histogram), make_plan(e, stream_ptr));
    e->launches += 1;
    return err == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

static LaunchPlan make_plan(const JfgpuEngine *e, void *stream_ptr) {
    LaunchPlan plan;
    plan.stream = static_cast<cudaStream_t>(stream_ptr);
    plan.warps = e->block_warps;
    plan.refine_limit = e->refine_limit;
    plan.groups = e->groups;
    plan.group_streams = e->groups > 1 ? const_cast<cudaStream_t *>(e->group_streams) : nullptr;
    plan.fork = e->fork;
    plan.join = const_cast<cudaEvent_t *>(e->join);
    plan.clock = e->clock;
    plan.graphs = e->graphs;
    return plan;
}

int jfgpu_chains_init(JfgpuEngine *e, const JfgpuBuffers *b, void *stream_ptr) {
    if (!buffers_ok(e, b)) return JFGPU_ERROR_ARGUMENT;
    cudaError_t err = launch_init(e->view, (long long)e->chains.size(), *b, make_plan(e, stream_ptr));
    e->launches += 1;
    return err == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

int jfgpu_chains_run(JfgpuEngine *e, const JfgpuBuffers *b, int64_t first, int64_t count, int64_t max_events,
                     double stop_q, double stop_r, int32_t mode, JfgpuEvent *log, int64_t log_capacity,
                     void *stream_ptr) {
    if (!buffers_ok(e, b) || first < 0 || count < 0 || first + count > (int64_t)e->chains.size() || max_events < 0 ||
        (mode != JFGPU_MODE_EXACT && mode != JFGPU_MODE_MIXED) || (log && log_capacity <= 0))
        return JFGPU_ERROR_ARGUMENT;
    if (count == 0 || max_events == 0) return JFGPU_OK;
    int potential = e->chains[first].potential, far = e->chains[first].far;
    for (int64_t c = first + 1; c < first + count && potential >= 0; ++c)
        if (e->chains[c].potential != potential || e->chains[c].far != far) potential = far = -1;
    long long launches = 0;
    cudaError_t err = launch_run(e->view, *b, first, count, max_events, stop_q, stop_r, mode, log, log_capacity,
                                 potential, far, e->refine_lists, e->refined, e->refine_queue, e->far_ahead,
                                 e->settle,
                                 (long long)e->chains.size(), make_plan(e, stream_ptr), &launches);
    e->launches += launches;
    return err == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

}  // extern "C"
