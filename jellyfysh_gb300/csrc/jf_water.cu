// jf_water.cu -- batched chains of flexible water: one warp per chain, the event loop on the device.
//
// Per event the lanes share the candidates of the active unit: every lane takes the other molecules lane,
// lane + 32, ... (the Coulomb factor of the two molecules: three bounded displacements; Lennard-Jones when the active
// unit is an oxygen), lanes 0-2 the bonds within the active molecule; a warp argmin over (time, kind, target) picks
// the event.  The out-state of a Coulomb event needs up to nine merged-image Coulomb derivatives: lanes 0-2 take the
// active unit against the three target units, lanes 3-8 the other two local units against them, all at once; every
// lane then runs the same thinning and lifting arithmetic (jf_composite.cuh) on the gathered values.  FP64 with the
// reference's arithmetic throughout; the random numbers are the keyed draws of (chain, event, kind, target).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "jf_composite.cuh"
#include "jf_engine.cuh"

namespace jf {

struct WaterModel {
    CompositeModel coulomb;  // units 3
    MH oh, hh, lj;
    double beta, chain_time, speed, length;
    int molecules, initial_active, initial_direction;
    uint64_t seed;
};

struct WaterArgs {
    WaterModel w;
    double *positions;
    const double *charges;
    JfgpuWaterState *state;
    JfgpuEvent *log;
    int64_t chains, first_chain, events;
};

struct WaterCand {
    double q, r;
    int kind, target;
};

// the earliest time; on equal times the lower kind, then the lower target (as the oracle orders candidates)
__device__ inline bool water_better(const WaterCand &a, const WaterCand &b) {
    if (time_lt(a.q, a.r, b.q, b.r)) return true;
    if (time_lt(b.q, b.r, a.q, a.r)) return false;
    if (a.kind != b.kind) return a.kind < b.kind;
    return a.target < b.target;
}

__device__ inline void water_offer(WaterCand &best, double ts_q, double ts_r, double dt, int kind, int target) {
    if (isinf(dt) && dt > 0) return;  // HeapScheduler.push_event ignores infinite times
    WaterCand c;
    time_add(ts_q, ts_r, dt, c.q, c.r);
    c.kind = kind;
    c.target = target;
    if (water_better(c, best)) best = c;
}

__device__ inline int water_new_active(const WaterModel &w, uint64_t key, uint64_t event) {
    const int molecule = (int)randbelow(draw(key, event, kRngNewActive, 0), (uint32_t)w.molecules);
    const int unit = (int)randbelow(draw(key, event, kRngNewActive, 1), 3u);
    return 3 * molecule + unit;
}

constexpr unsigned kFull = 0xffffffffu;

__device__ inline double shfl_double(double v, int lane) { return __shfl_sync(kFull, v, lane); }

__global__ void water_init_kernel(WaterModel w, JfgpuWaterState *state, int64_t chains, int64_t first_chain) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= chains) return;
    const uint64_t key = chain_key(w.seed, (uint64_t)(first_chain + c));
    JfgpuWaterState s;
    memset(&s, 0, sizeof(s));
    s.active = w.initial_active;
    s.direction = w.initial_direction;
    time_add(0.0, 0.0, time_sub(0.0, 0.0, 0.0, 0.0) + w.chain_time, s.eoc_q, s.eoc_r);
    s.eoc_new_active = water_new_active(w, key, 0);
    state[c] = s;
}

__global__ void water_kernel(WaterArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t chain = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (chain >= a.chains) return;  // whole warps
    const WaterModel &w = a.w;
    const int M = w.molecules;
    const uint64_t key = chain_key(w.seed, (uint64_t)(a.first_chain + chain));
    double *pos = a.positions + (size_t)chain * 9 * M;
    const double *charge = a.charges;
    JfgpuWaterState s = a.state[chain];
    for (int64_t step = 0; step < a.events && s.status == JFGPU_STATUS_OK; ++step) {
        const int act = s.active, m = act / 3, t = act % 3, d = s.direction;
        const uint64_t ev = (uint64_t)s.events;
        double velocity[3] = {0.0, 0.0, 0.0};
        velocity[d] = w.speed;
        double pa[3];
        for (int c = 0; c < 3; ++c) pa[c] = pos[3 * act + c];
        const double ca = charge[act];
        WaterCand best;
        best.q = INFINITY;
        best.r = INFINITY;
        best.kind = 1 << 30;
        best.target = 1 << 30;
        int st = JFGPU_STATUS_OK;
        for (int other = lane; other < M && !st; other += 32) {
            if (other == m) continue;
            double du[3], dt = 0.0;
            for (int j = 0; j < 3; ++j)
                du[j] = expovariate(draw(key, ev, kRngComposite, (uint32_t)(3 * other + j)), w.beta);
            st = composite_event_time(w.coulomb, velocity, pa, ca, pos + 9 * other, charge + 3 * other, du, dt);
            if (st) break;
            water_offer(best, s.time_q, s.time_r, dt, JFGPU_EV_COMPOSITE, other);
            if (t == 1) {
                const int b = 3 * other + 1;
                double sep[3], value;
                periodic_separation(pa, pos + 3 * b, w.length, sep);
                const double u = expovariate(draw(key, ev, kRngPair, (uint32_t)b), w.beta);
                st = mh_std_displacement(w.lj, d, sep, u, value);
                if (st) break;
                water_offer(best, s.time_q, s.time_r, value / w.speed, JFGPU_EV_PAIR, b);
            }
        }
        if (!st && lane < 3 && lane != t) {
            const int b = 3 * m + lane;
            const MH &bond = (t == 1 || lane == 1) ? w.oh : w.hh;
            double sep[3], value;
            periodic_separation(pa, pos + 3 * b, w.length, sep);
            const double u = expovariate(draw(key, ev, kRngPair, (uint32_t)b), w.beta);
            st = mh_std_displacement(bond, d, sep, u, value);
            if (!st) water_offer(best, s.time_q, s.time_r, value / w.speed, JFGPU_EV_BOND, b);
        }
        const unsigned failed = __ballot_sync(kFull, st != JFGPU_STATUS_OK);
        if (failed) {
            s.status = __shfl_sync(kFull, st, __ffs(failed) - 1);
            break;
        }
        for (int offset = 16; offset > 0; offset >>= 1) {
            WaterCand o;
            o.q = __shfl_xor_sync(kFull, best.q, offset);
            o.r = __shfl_xor_sync(kFull, best.r, offset);
            o.kind = __shfl_xor_sync(kFull, best.kind, offset);
            o.target = __shfl_xor_sync(kFull, best.target, offset);
            if (water_better(o, best)) best = o;
        }
        {
            WaterCand e;
            e.q = s.eoc_q;
            e.r = s.eoc_r;
            e.kind = JFGPU_EV_END_OF_CHAIN;
            e.target = s.eoc_new_active;
            if (water_better(e, best)) best = e;
        }
        // commit: time slice of the active unit (every lane computes the same position; lane 0 stores it)
        {
            const double dt = time_sub(best.q, best.r, s.time_q, s.time_r);
            for (int c = 0; c < 3; ++c) pa[c] = py_mod(pa[c] + velocity[c] * dt, w.length);
            if (lane == 0)
                for (int c = 0; c < 3; ++c) pos[3 * act + c] = pa[c];
            s.time_q = best.q;
            s.time_r = best.r;
        }
        __syncwarp();
        int accepted = 1;
        if (best.kind == JFGPU_EV_BOND || best.kind == JFGPU_EV_PAIR) {
            s.active = best.target;
            if (best.kind == JFGPU_EV_BOND) ++s.bond_events; else ++s.lj_events;
        } else if (best.kind == JFGPU_EV_COMPOSITE) {
            const int other = best.target;
            const double *locals = pos + 9 * m, *targets = pos + 9 * other;
            // lanes 0-2: the active unit against target unit `lane` (bound and potential); lanes 3-8: local unit
            // i (the (lane - 3) / 3-th unit other than the active one) against target unit (lane - 3) % 3
            double mine_bound = 0.0, mine_pair = 0.0;
            if (lane < 3) {
                double sep[3];
                periodic_separation(pa, targets + 3 * lane, w.length, sep);
                mine_bound = bound_derivative(w.coulomb, d, w.speed, sep, ca, charge[3 * other + lane]);
                mine_pair = coulomb_derivative(w.coulomb, d, w.speed, sep, ca, charge[3 * other + lane]);
            } else if (lane < 9) {
                const int k = (lane - 3) / 3, j = (lane - 3) % 3;
                const int i = k < t ? k : k + 1;
                double sep[3];
                periodic_separation(locals + 3 * i, targets + 3 * j, w.length, sep);
                mine_pair = coulomb_derivative(w.coulomb, d, w.speed, sep, charge[3 * m + i], charge[3 * other + j]);
            }
            double bound[3], pair[3], cross[9], target_factor[3];
            for (int j = 0; j < 3; ++j) {
                bound[j] = shfl_double(mine_bound, j);
                pair[j] = shfl_double(mine_pair, j);
            }
            for (int k = 0; k < 2; ++k) {
                const int i = k < t ? k : k + 1;
                for (int j = 0; j < 3; ++j) cross[i * 3 + j] = shfl_double(mine_pair, 3 + 3 * k + j);
            }
            for (int j = 0; j < 3; ++j) cross[t * 3 + j] = 0.0;  // the active row is not read
            double draws[3];
            draws[0] = uniform53(draw(key, ev, kRngThin, 0));
            draws[1] = uniform53(draw(key, ev, kRngLift, 0));
            draws[2] = draws[1];
            double bounding_rate, event_rate;
            ++s.composite_events;
            accepted = 0;
            if (composite_thinning(w.coulomb, JFGPU_DRAW_UNIT, bound, pair, draws, target_factor, bounding_rate,
                                   event_rate)) {
                int new_active = -1;
                st = composite_lifting(w.coulomb, JFGPU_DRAW_UNIT, t, m < other, event_rate, target_factor, cross,
                                       draws, new_active);
                if (st) {
                    s.status = st;
                    break;
                }
                accepted = 1;
                ++s.composite_accepted;
                s.active = new_active < 3 ? 3 * m + new_active : 3 * other + (new_active - 3);
            }
        } else if (best.kind == JFGPU_EV_END_OF_CHAIN) {
            s.direction = (s.direction + 1) % 3;
            s.active = best.target;
            time_add(s.time_q, s.time_r, time_sub(s.time_q, s.time_r, s.time_q, s.time_r) + w.chain_time, s.eoc_q,
                     s.eoc_r);
            s.eoc_new_active = water_new_active(w, key, ev + 1);
            ++s.eoc_events;
        } else {
            s.status = JFGPU_STATUS_ASSERTION;
            break;
        }
        if (lane == 0 && a.log) {
            JfgpuEvent e;
            e.kind = best.kind;
            e.moved = act;
            e.target = best.target;
            e.new_active = s.active;
            e.new_direction = s.direction;
            e.accepted = accepted;
            e.time_q = best.q;
            e.time_r = best.r;
            e.x = pa[0];
            e.y = pa[1];
            e.z = pa[2];
            a.log[chain * a.events + step] = e;
        }
        ++s.events;
    }
    if (lane == 0) a.state[chain] = s;
}

struct WaterHandle {
    WaterModel model;
    double *fourier = nullptr;
    int device = -1;
};

}  // namespace jf

using namespace jf;

extern "C" int jfgpu_water_create(const JfgpuWaterDesc *desc, void **water) {
    if (!desc || !water) return JFGPU_ERROR_ARGUMENT;
    *water = nullptr;
    if (desc->molecules < 2 || desc->molecules > 4096 || !(desc->system_length > 0.0) || !(desc->beta > 0.0) ||
        !(desc->speed > 0.0) || !(desc->chain_time > 0.0) || desc->initial_active < 0 ||
        desc->initial_active >= 3 * desc->molecules || desc->initial_direction < 0 || desc->initial_direction > 2 ||
        desc->lifting < JFGPU_LIFTING_INSIDE_FIRST || desc->lifting > JFGPU_LIFTING_RATIO ||
        desc->fourier_cutoff < 0 || desc->position_cutoff < 0 || !(desc->alpha > 0.0))
        return JFGPU_ERROR_ARGUMENT;
    WaterHandle *h = new WaterHandle();
    if (cudaGetDevice(&h->device) != cudaSuccess) {
        delete h;
        return JFGPU_ERROR_CUDA;
    }
    std::vector<double> table = fourier_table(desc->fourier_cutoff, desc->alpha, desc->system_length);
    if (cudaMalloc((void **)&h->fourier, table.size() * sizeof(double)) != cudaSuccess) {
        delete h;
        return JFGPU_ERROR_ALLOCATION;
    }
    if (cudaMemcpy(h->fourier, table.data(), table.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(h->fourier);
        delete h;
        return JFGPU_ERROR_CUDA;
    }
    WaterModel &w = h->model;
    w.coulomb.mic = make_mic(desc->fourier_cutoff, desc->position_cutoff, desc->alpha, desc->system_length,
                             h->fourier);
    w.coulomb.coulomb_prefactor = desc->coulomb_prefactor;
    w.coulomb.bound_prefactor = desc->bound_prefactor;
    w.coulomb.system_length = desc->system_length;
    w.coulomb.units = 3;
    w.coulomb.lifting = desc->lifting;
    w.oh = make_displaced(desc->oh_r0, 2, desc->oh_prefactor);
    w.hh = make_displaced(desc->hh_r0, 2, desc->hh_prefactor);
    w.lj = make_lj(desc->lj_prefactor, desc->lj_sigma);
    w.beta = desc->beta;
    w.chain_time = desc->chain_time;
    w.speed = desc->speed;
    w.length = desc->system_length;
    w.molecules = desc->molecules;
    w.initial_active = desc->initial_active;
    w.initial_direction = desc->initial_direction;
    w.seed = desc->seed;
    *water = h;
    return JFGPU_OK;
}

extern "C" void jfgpu_water_destroy(void *water) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h) return;
    if (h->fourier) cudaFree(h->fourier);
    delete h;
}

extern "C" int jfgpu_water_init(void *water, JfgpuWaterState *state, int64_t chains, int64_t first_chain,
                                void *stream) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h || chains < 0 || first_chain < 0) return JFGPU_ERROR_ARGUMENT;
    if (chains == 0) return JFGPU_OK;
    if (!state) return JFGPU_ERROR_ARGUMENT;
    const int threads = 128;
    water_init_kernel<<<(unsigned)((chains + threads - 1) / threads), threads, 0, static_cast<cudaStream_t>(stream)>>>(
        h->model, state, chains, first_chain);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

extern "C" int jfgpu_water_run(void *water, double *positions, const double *charges, JfgpuWaterState *state,
                               int64_t chains, int64_t first_chain, int64_t events, JfgpuEvent *log,
                               int32_t warps_per_block, void *stream) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h || chains < 0 || first_chain < 0 || events < 0 || warps_per_block < 0 || warps_per_block > 8)
        return JFGPU_ERROR_ARGUMENT;
    if (chains == 0 || events == 0) return JFGPU_OK;
    if (!positions || !charges || !state) return JFGPU_ERROR_ARGUMENT;
    const int warps = warps_per_block ? warps_per_block : 1;
    WaterArgs a;
    a.w = h->model;
    a.positions = positions;
    a.charges = charges;
    a.state = state;
    a.log = log;
    a.chains = chains;
    a.first_chain = first_chain;
    a.events = events;
    const int64_t blocks = (chains + warps - 1) / warps;
    water_kernel<<<(unsigned)blocks, 32 * warps, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}
