// jf_water.cu -- batched chains of flexible water: one block per chain, the event loop on the device.
//
// Per event the threads share the candidate items of the active unit: the bounded displacement against every unit
// of every other molecule (the Coulomb factors), Lennard-Jones against every other oxygen when the active unit is an
// oxygen, the two bonds within the molecule; a block argmin over (time, kind, target) picks the event.  The
// out-state of a Coulomb event needs three merged-image Coulomb derivatives for the thinning and six more for the
// lifting; each is shared by one warp (mic_x_warp: the images and Fourier rows of the sum spread over the lanes), the
// warps take different ones, and thread 0 runs the thinning and lifting arithmetic (jf_composite.cuh).  FP64 with
// the reference's arithmetic throughout (the merged-image sums in another order of additions); in the mixed mode the
// thinning first tries FP32 sums with an error bound.  The random numbers are the keyed draws of (chain, event,
// kind, target).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "jf_composite.cuh"
#include "jf_engine.cuh"
#include "jf_screen.cuh"

namespace jf {

// the molecular cells of a water model: cuboid periodic cells of the root units, the nearby cells of the neighbour
// layers and the molecular cell veto's bound and Walker tables
struct WaterCells {
    int m, ncells, n_off;
    int keep_pairs;           // the bond and Lennard-Jones candidates outlive a cell boundary
    int far;                  // JFGPU_FAR_CELL_VETO, or JFGPU_FAR_CELL_BOUNDING (a factor for every occupied far cell)
    double dipole_charge;     // the estimator's dipole charge (the cell-bounding charge factor)
    int offsets[32];          // the distinct residues of -layers .. layers modulo m, ascending
    double side;              // L / m: position_to_cell is int(x / side) along every axis
    double inv_side;          // 1 / side, the first guess of int(x / side)
    double root_speed;        // the active root unit's velocity component: the speed times the leaf's weight 1/3
    const double *cell_min;   // [m] exact lower cell bounds along an axis
    const double *cell_max;   // [m] exact upper cell bounds along an axis
    const int16_t *tra;       // [m * m] translate along one axis, [a * m + b]
    const int16_t *rel;       // [m * m] relative_cell along one axis, [a * m + b]
    const double *bound_upper, *bound_lower;  // [ncells][3] upper and negated lower bounds
    WalkerDev walker[2][3];   // [upper / lower][direction]
};

struct WaterModel {
    CompositeModel coulomb;  // units 3
    MH oh, hh, lj;
    double beta, chain_time, speed, length;
    float beta32, speed32, length32;
    LJ32 lj32;            // the Lennard-Jones constants of the FP32 screen
    float margin32;       // rounding scale of FP32 separations, 16 L 2^-24
    int molecules, initial_active, initial_direction, mode;
    uint64_t seed;
    int cells_on;         // the molecular cells are attached (jfgpu_water_set_cells)
    WaterCells cells;
};

struct WaterArgs {
    WaterModel w;
    double *positions;
    const double *charges;
    JfgpuWaterState *state;
    JfgpuEvent *log;
    int64_t chains, first_chain, events;
    double stop_q, stop_r;  // stop time (inf: none)
    // molecular cells
    double *roots;          // [chains][molecules][3]
    int32_t *occ;           // [chains][cells]
    int32_t *sur;           // [chains][molecules]
    JfgpuWaterCellState *cell_state;
    double *root_log;       // [chains][events][3] or null
};

struct WaterCand {
    double q, r;
    int kind, target;
};

// the earliest time; on equal times the lower kind, then the lower target (as the oracle orders candidates).  The
// quotient and remainder of a time are non-negative (never -0.0, as Python's divmod gives) or +inf, so their IEEE
// bit patterns order as the values do: the comparison runs on integers, off GB300's scarce FP64 pipe.
__device__ inline bool water_better(const WaterCand &a, const WaterCand &b) {
    const unsigned long long aq = (unsigned long long)__double_as_longlong(a.q);
    const unsigned long long bq = (unsigned long long)__double_as_longlong(b.q);
    if (aq != bq) return aq < bq;
    const unsigned long long ar = (unsigned long long)__double_as_longlong(a.r);
    const unsigned long long br = (unsigned long long)__double_as_longlong(b.r);
    if (ar != br) return ar < br;
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

constexpr int kMaxWarps = 8;

// candidate items of an event at most: Coulomb items in three warp-padded groups, Lennard-Jones, two bonds
__host__ __device__ inline int water_items_max(int molecules) {
    return 3 * (((molecules - 1) + 31) & ~31) + (molecules - 1) + 2;
}

// chunks of 32 items (one warp's share of a round)
__host__ __device__ inline int water_chunks_max(int molecules) { return (water_items_max(molecules) + 31) >> 5; }

// candidate items of an event of the kernel with molecular cells at most: the Coulomb items of the nearby and
// surplus molecules in three warp-padded groups, the far cell-bounding items padded to whole warps, Lennard-Jones, two
// bonds (the target molecules of the two lists together are at most molecules - 1)
__host__ __device__ inline int water_cells_items_max(int molecules) {
    return 4 * (((molecules - 1) + 31) & ~31) + (molecules - 1) + 2;
}

// dynamic shared memory of the kernel with molecular cells: per-item lower bounds (float), the item list (int), the
// taken count of every chunk of 32 items (int), the target list [molecules], the screen's prefactors [3 molecules] and
// the far target list [molecules]
__host__ inline size_t water_cells_shared_bytes(int molecules) {
    const int items = water_cells_items_max(molecules);
    return (size_t)items * (sizeof(float) + sizeof(int)) + (size_t)((items + 31) >> 5) * sizeof(int) +
           sizeof(int) * 5 * (size_t)molecules;
}

// per-item lower bounds (float), the item list (int), the taken count of every chunk (int)
__host__ inline size_t water_shared_bytes(int molecules) {
    const int items = water_items_max(molecules);
    return (size_t)items * sizeof(float) + (size_t)items * sizeof(int) +
           (size_t)water_chunks_max(molecules) * sizeof(int);
}

// the bounded displacement of the active unit against unit j of molecule `other`: the Coulomb factor of the two
// molecules takes the smallest over the three; as time_add does not decrease with the displacement, the smallest of
// the three times is the same time (two_composite_object_summed_bounding_potential_event_handler.py:119-150)
__device__ inline void coulomb_unit_exact(const WaterModel &w, const double *pos, const double *charge, uint64_t key,
                                          uint64_t ev, int other, int j, int d, const double *pa, double ca,
                                          double ts_q, double ts_r, WaterCand &best) {
    const int b = 3 * other + j;
    const double du = expovariate(draw(key, ev, kRngComposite, (uint32_t)b), w.beta);
    double sep[3], p[3];
    periodic_separation(pa, pos + 3 * b, w.length, sep);
    permute3(sep, d, p);
    const double value = ipcb_x_displacement(w.coulomb.bound_prefactor * ca * charge[b], p[0], p[1], p[2], du,
                                             w.length) / w.speed;
    water_offer(best, ts_q, ts_r, value, JFGPU_EV_COMPOSITE, other);
}

// pair item k of the active unit 3 m + t: Lennard-Jones against the oxygen of another molecule for k < n_lj, else
// one of the two bonds within the molecule (two_leaf_unit_event_handler.py:98-138)
__device__ inline int pair_item_exact(const WaterModel &w, const double *pos, uint64_t key, uint64_t ev, int k,
                                      int n_lj, int m, int t, int d, const double *pa, double ts_q, double ts_r,
                                      WaterCand &best) {
    int b, kind;
    const MH *h;
    if (k < n_lj) {
        const int other = k + (k >= m);
        b = 3 * other + 1;
        h = &w.lj;
        kind = JFGPU_EV_PAIR;
    } else {
        const int u = (k - n_lj) + ((k - n_lj) >= t);  // the two other units of the molecule
        b = 3 * m + u;
        h = (t == 1 || u == 1) ? &w.oh : &w.hh;
        kind = JFGPU_EV_BOND;
    }
    double sep[3];
    periodic_separation(pa, pos + 3 * b, w.length, sep);
    const double du = expovariate(draw(key, ev, kRngPair, (uint32_t)b), w.beta);
    double value;
    JF_TRY(mh_std_displacement(*h, d, sep, du, value));
    water_offer(best, ts_q, ts_r, value / w.speed, kind, b);
    return JFGPU_STATUS_OK;
}

// one candidate item of the event: the bounded displacement of the active unit against one unit of another molecule,
// Lennard-Jones against another oxygen, or a bond within the molecule.  Returns a status; the candidate is offered
// to best.
__device__ inline int water_item(const WaterModel &w, const double *pos, const double *charge, uint64_t key,
                                 uint64_t ev, int item, int m, int t, int d, const double *pa, double ca, double ts_q,
                                 double ts_r, WaterCand &best) {
    const int M = w.molecules;
    // Coulomb items grouped by target unit type (hydrogen, oxygen, hydrogen), each group padded to whole warps, so
    // that a warp solves displacements of one charge sign (one branch of the inversion)
    const int group = ((M - 1) + 31) & ~31;
    const int n_coulomb = 3 * group, n_lj = t == 1 ? M - 1 : 0;
    if (item < n_coulomb) {
        const int j = item / group;
        int other = item % group;
        if (other >= M - 1) return JFGPU_STATUS_OK;  // padding
        other += other >= m;
        coulomb_unit_exact(w, pos, charge, key, ev, other, j, d, pa, ca, ts_q, ts_r, best);
        return JFGPU_STATUS_OK;
    }
    return pair_item_exact(w, pos, key, ev, item - n_coulomb, n_lj, m, t, d, pa, ts_q, ts_r, best);
}

__device__ inline void coulomb_unit_screen(const WaterModel &w, const double *pos, const double *charge,
                                           uint64_t key, uint64_t ev, int other, int j, int d, const double *pa,
                                           double ca, float &time, float &error, bool &unsafe,
                                           const float *pp32 = nullptr);

// FP32 lower bound of the time of bond k of the active unit 3 m + t (the k-th of the two other units of its
// molecule): a bond k (|s| - r0)^2 along the motion has |d|s|/dx| <= 1, so the potential rises at most at
// 2 k (a + x) with a = ||s| - r0| after a displacement x, and a rise du takes at least
// (du / k) / (a + sqrt(a^2 + du / k)); computed with every rounding towards a smaller value.  It bounds the bond's
// time from below only.
__device__ inline void bond_unit_screen(const WaterModel &w, const double *pos, uint64_t key, uint64_t ev, int m,
                                        int t, int k, const double *pa, float &time, bool &unsafe) {
    const int u = k + (k >= t);
    const int b = 3 * m + u;
    const MH &bond = (t == 1 || u == 1) ? w.oh : w.hh;
    bool flag = false;
    const float du = expovariate32(draw(key, ev, kRngPair, (uint32_t)b), 1.0f / w.beta32, flag);
    double sep[3];
    periodic_separation(pa, pos + 3 * b, w.length, sep);
    const float r = sqrtf((float)(sep[0] * sep[0] + sep[1] * sep[1] + sep[2] * sep[2]));
    const float a = fabsf(r - (float)bond.r0) * (1.f + 0x1p-16f) + 0x1p-20f * (float)bond.r0;
    const float ratio = du * (1.f - 0x1p-16f) / (float)(bond.prefactor * (1.0 + 0x1p-20));
    time = ratio / (a + sqrtf(a * a + ratio)) * (1.f - 0x1p-16f) / w.speed32;
    unsafe = flag || !(time >= 0.f);
}

// FP32 screen of Lennard-Jones against the oxygen of molecule `other` (over the speed): the FP32 screen of the
// atomic engine, within 2^-13 relative plus its absolute margin unless flagged; a pair without an event (U + du
// stays below zero) screens to an infinite time that is safe
__device__ inline void lj_unit_screen(const WaterModel &w, const double *pos, uint64_t key, uint64_t ev, int other,
                                      int d, const double *pa, float &time, float &error, bool &unsafe) {
    const int b = 3 * other + 1;
    bool flag = false;
    const float du = expovariate32(draw(key, ev, kRngPair, (uint32_t)b), 1.0f / w.beta32, flag);
    double sep64[3];
    periodic_separation(pa, pos + 3 * b, w.length, sep64);
    float sep[3] = {(float)sep64[0], (float)sep64[1], (float)sep64[2]};
    int path;
    time = lj_screen(w.lj32, d, w.speed32, sep, du, w.margin32, flag, path);
    error = 0x1p-11f * fabsf(time) + w.length32 * 0x1p-17f / w.speed32;
    unsafe = flag || isinf(time);
    if (isinf(time) && !flag) {
        unsafe = false;
        time = INFINITY;
        error = 0.f;
    }
}

// FP32 screen of a candidate item, in displacements over the speed: the Coulomb items solve the bound's inversion
// in FP32 with an error bound (ipcb_x_displacement32), the Lennard-Jones items take the FP32 screen of the atomic
// engine; a bond gets only a lower bound of its time (lower_only: it does not bound the earliest time).  unsafe:
// the screen cannot decide, the item goes to FP64.
__device__ inline void water_screen(const WaterModel &w, const double *pos, const double *charge, uint64_t key,
                                   uint64_t ev, int item, int m, int t, int d, const double *pa, double ca,
                                   float &time, float &error, bool &unsafe, bool &lower_only) {
    const int M = w.molecules;
    const int group = ((M - 1) + 31) & ~31;
    unsafe = false;
    lower_only = false;
    time = 0.f;
    error = 0.f;
    if (item >= 3 * group + (t == 1 ? M - 1 : 0)) {
        bond_unit_screen(w, pos, key, ev, m, t, item - 3 * group - (t == 1 ? M - 1 : 0), pa, time, unsafe);
        lower_only = true;
        return;
    }
    if (item >= 3 * group) {
        // Lennard-Jones against another oxygen (only listed when the active unit is an oxygen)
        int other = item - 3 * group;
        other += other >= m;
        lj_unit_screen(w, pos, key, ev, other, d, pa, time, error, unsafe);
        return;
    }
    const int j = item / group;
    int other = item % group;
    if (other >= M - 1) {
        time = INFINITY;  // padding
        return;
    }
    other += other >= m;
    coulomb_unit_screen(w, pos, charge, key, ev, other, j, d, pa, ca, time, error, unsafe);
}

// FP32 screen of the bounded displacement of the active unit against unit j of molecule `other` (over the speed),
// with its error bound; unsafe: the screen cannot decide
// pp32: the FP32 prefactors (float)(bound prefactor * active charge * charge[b]) of every unit b, or null to compute
// the unit's here
__device__ inline void coulomb_unit_screen(const WaterModel &w, const double *pos, const double *charge,
                                           uint64_t key, uint64_t ev, int other, int j, int d, const double *pa,
                                           double ca, float &time, float &error, bool &unsafe, const float *pp32) {
    const int b = 3 * other + j;
    // du = -log(1 - u) / beta of the FP64 draw u = n 2^-53 (uniform53): log1pf(-u) below u = 1/2 (u rounded to
    // FP32 moves -log(1 - u) by at most 2 units of 2^-24 relative there), logf of the exact 1 - u = (2^53 - n) 2^-53
    // from u = 1/2 (the rounding of the argument moves the logarithm by 2^-24, at least ln 2 in size); with the
    // errors of log1pf or logf, beta in FP32 and the division, within 8 units, taken as 24
    const uint64_t n = draw(key, ev, kRngComposite, (uint32_t)b) >> 11;
    const float du = n < (1ull << 52) ? -log1pf(-(float)n * 0x1p-53f) / w.beta32
                                      : -logf((float)((1ull << 53) - n) * 0x1p-53f) / w.beta32;
    const float du_error = 24.f * 0x1p-24f * du;
    double sep[3], p[3];
    periodic_separation(pa, pos + 3 * b, w.length, sep);
    permute3(sep, d, p);
    float value_error;
    const float pp = pp32 ? pp32[b] : (float)(w.coulomb.bound_prefactor * ca * charge[b]);
    const float value = ipcb_x_displacement32(pp, (float)p[0],
                                              (float)p[1], (float)p[2], du, du_error, w.length32, value_error,
                                              unsafe);
    time = value / w.speed32;
    error = value_error / w.speed32 + 0x1p-23f * fabsf(time);
}

__device__ inline void shuffle_better(WaterCand &best, int offset) {
    WaterCand o;
    o.q = __shfl_xor_sync(kFull, best.q, offset);
    o.r = __shfl_xor_sync(kFull, best.r, offset);
    o.kind = __shfl_xor_sync(kFull, best.kind, offset);
    o.target = __shfl_xor_sync(kFull, best.target, offset);
    if (water_better(o, best)) best = o;
}

// One block of `warps` warps advances one chain.  Candidate items are spread over all threads; the argmin goes
// through warp shuffles and shared memory; the merged-image sums of a Coulomb out-state go to different warps.
// Decisions that every thread can take from shared values (the bound of the screen, the list offsets, the winner,
// the thinning) are taken by every thread, so that an event crosses few block barriers: after the screen, after the
// chunk counts, after the list, after the argmin, after the out-state sums, and at the end of the event.  Thread 0
// alone updates the chain state, after the last read of it by the other threads (the state of the event is read
// into registers at its start).  At most 128 registers a thread, so that five blocks of 96 threads (the default
// three warps) share an SM and 512 chains run in one wave on the 152 SMs.
__global__ void __launch_bounds__(256, 2) water_kernel(WaterArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    const int64_t chain = blockIdx.x;
    if (chain >= a.chains) return;  // whole blocks
    const WaterModel &w = a.w;
    const int M = w.molecules;
    const uint64_t key = chain_key(w.seed, (uint64_t)(a.first_chain + chain));
    double *pos = a.positions + (size_t)chain * 9 * M;
    const double *charge = a.charges;
    __shared__ JfgpuWaterState s;
    __shared__ WaterCand warp_best[kMaxWarps];
    __shared__ float warp_upper[kMaxWarps];
    // per-item lower bounds of the screen, the list of items for the FP64 pass and the taken count of every chunk of
    // 32 items (dynamic shared memory)
    extern __shared__ float dynamic[];
    float *lower = dynamic;
    int *list = reinterpret_cast<int *>(dynamic + water_items_max(M));
    int *chunk_count = list + water_items_max(M);
    __shared__ int status;
    __shared__ double bound[3], pair[3], cross[9];
    __shared__ float pair32[3], error32[3], bound32[3];
    if (threadIdx.x == 0) {
        s = a.state[chain];
        s.stopped = 0;
        status = JFGPU_STATUS_OK;
    }
    __syncthreads();
    for (int64_t step = 0; step < a.events && s.status == JFGPU_STATUS_OK; ++step) {
        const int act = s.active, m = act / 3, t = act % 3, d = s.direction;
        const uint64_t ev = (uint64_t)s.events;
        const double ts_q = s.time_q, ts_r = s.time_r;
        WaterCand eoc;
        eoc.q = s.eoc_q;
        eoc.r = s.eoc_r;
        eoc.kind = JFGPU_EV_END_OF_CHAIN;
        eoc.target = s.eoc_new_active;
        double pa[3];
        for (int c = 0; c < 3; ++c) pa[c] = pos[3 * act + c];
        const double ca = charge[act];
        WaterCand best;
        best.q = INFINITY;
        best.r = INFINITY;
        best.kind = 1 << 30;
        best.target = 1 << 30;
        const int items = 3 * (((M - 1) + 31) & ~31) + (t == 1 ? M - 1 : 0) + 2;
        int st = JFGPU_STATUS_OK, refined = 3 * (M - 1) + (t == 1 ? M - 1 : 0) + 2;
        if (w.mode == JFGPU_MODE_MIXED) {
            // phase A: FP32 screen of every item; lower[item] = the earliest time the item may reach (-inf where
            // the screen cannot decide), the bound = the smallest time that some candidate surely reaches (a screened
            // time plus its error bound, or the end of chain); the differences round outwards, towards a smaller
            // lower bound and a larger bound, so that an item is listed whenever its exact time may come first
            float mine = INFINITY;
            for (int item = threadIdx.x; item < items; item += blockDim.x) {
                float t32, e32;
                bool unsafe, lower_only;
                water_screen(w, pos, charge, key, ev, item, m, t, d, pa, ca, t32, e32, unsafe, lower_only);
                lower[item] = unsafe ? -INFINITY : __fsub_rd(t32, e32);
                if (!unsafe && !lower_only) mine = fminf(mine, __fadd_ru(t32, e32));
            }
            for (int offset = 16; offset > 0; offset >>= 1) mine = fminf(mine, __shfl_xor_sync(kFull, mine, offset));
            if (lane == 0) warp_upper[warp] = mine;
            __syncthreads();
            float bound_time = __double2float_ru(time_sub(eoc.q, eoc.r, ts_q, ts_r));
            for (int k = 0; k < warps; ++k) bound_time = fminf(bound_time, warp_upper[k]);
            // the items that may come first, listed in item order (Coulomb items by unit type, then Lennard-Jones,
            // then bonds) so that each warp of the FP64 pass follows one kind of solve: the taken count of every
            // chunk of 32 items, then (every warp scanning the counts) the items of the warp's chunks at their offsets
            const int chunks = (items + 31) >> 5, coulomb_chunks = (3 * (((M - 1) + 31) & ~31)) >> 5;
            for (int c = warp; c < chunks; c += warps) {
                const int item = 32 * c + lane;
                const unsigned votes = __ballot_sync(kFull, item < items && lower[item] <= bound_time);
                if (lane == 0) chunk_count[c] = __popc(votes);
            }
            __syncthreads();
            int taken = 0, coulomb_taken = 0;
            for (int g = 0; g < chunks; g += 32) {
                const int v = g + lane < chunks ? chunk_count[g + lane] : 0;
                int inclusive = v;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(kFull, inclusive, o);
                    if (lane >= o) inclusive += y;
                }
                const int before = taken + inclusive - v;  // items taken before chunk g + lane
                if (coulomb_chunks >= g && coulomb_chunks < g + 32)
                    coulomb_taken = __shfl_sync(kFull, before, coulomb_chunks - g);
                const int first = warp >= g ? warp : warp + ((g - warp + warps - 1) / warps) * warps;
                for (int c = first; c < g + 32 && c < chunks; c += warps) {
                    const int offset = __shfl_sync(kFull, before, c - g);
                    const int item = 32 * c + lane;
                    const bool take = item < items && lower[item] <= bound_time;
                    const unsigned votes = __ballot_sync(kFull, take);
                    if (take) list[offset + __popc(votes & ((1u << lane) - 1u))] = item;
                }
                taken += __shfl_sync(kFull, inclusive, 31);
            }
            const int bonds_taken = (lower[items - 2] <= bound_time) + (lower[items - 1] <= bound_time);
            const int lj_taken = taken - coulomb_taken - bonds_taken;
            __syncthreads();
            // phase B: the FP64 solve of the listed items; each kind of solve starts on a warp boundary, so that a
            // warp follows one kind (Coulomb, Lennard-Jones, bonds)
            const int lj_start = (coulomb_taken + 31) & ~31;
            const int bond_start = lj_start + ((lj_taken + 31) & ~31);
            for (int v = threadIdx.x; v < bond_start + bonds_taken && !st; v += blockDim.x) {
                int k = -1;
                if (v < coulomb_taken)
                    k = v;
                else if (v >= lj_start && v < lj_start + lj_taken)
                    k = coulomb_taken + (v - lj_start);
                else if (v >= bond_start)
                    k = coulomb_taken + lj_taken + (v - bond_start);
                if (k >= 0) st = water_item(w, pos, charge, key, ev, list[k], m, t, d, pa, ca, ts_q, ts_r, best);
            }
            refined = taken;
        } else {
            for (int item = threadIdx.x; item < items && !st; item += blockDim.x)
                st = water_item(w, pos, charge, key, ev, item, m, t, d, pa, ca, ts_q, ts_r, best);
        }
        if (st) status = st;  // any failing thread; all stop after the barrier
        for (int offset = 16; offset > 0; offset >>= 1) shuffle_better(best, offset);
        if (lane == 0) warp_best[warp] = best;
        __syncthreads();
        if (status != JFGPU_STATUS_OK) {
            if (threadIdx.x == 0) s.status = status;
            break;
        }
        // every thread takes the winner: the warps' best, the end of chain, the stop time (which wins ties)
        best = warp_best[0];
        for (int k = 1; k < warps; ++k)
            if (water_better(warp_best[k], best)) best = warp_best[k];
        if (water_better(eoc, best)) best = eoc;
        if (!isinf(a.stop_q) && !time_lt(best.q, best.r, a.stop_q, a.stop_r)) {
            // the end of the run: the active unit time-sliced to the stop time, no event
            if (threadIdx.x == 0) {
                const double dt = time_sub(a.stop_q, a.stop_r, ts_q, ts_r);
                for (int c = 0; c < 3; ++c)
                    pos[3 * act + c] = py_mod_near(pa[c] + (c == d ? w.speed : 0.0) * dt, w.length);
                s.time_q = a.stop_q;
                s.time_r = a.stop_r;
                s.stopped = 1;
            }
            break;
        }
        // commit: time slice of the active unit (every thread computes the same position; thread 0 stores it)
        {
            const double dt = time_sub(best.q, best.r, ts_q, ts_r);
            for (int c = 0; c < 3; ++c) pa[c] = py_mod_near(pa[c] + (c == d ? w.speed : 0.0) * dt, w.length);
        }
        int accepted = 1;
        if (best.kind == JFGPU_EV_COMPOSITE) {
            const int other = best.target;
            const double *locals = pos + 9 * m, *targets = pos + 9 * other;
            double draws[3];
            draws[0] = uniform53(draw(key, ev, kRngThin, 0));
            draws[1] = uniform53(draw(key, ev, kRngLift, 0));
            draws[2] = draws[1];
            // in the mixed mode, FP32 first: the merged-image sums (warp j for target unit j) and the bounding
            // derivatives, each with an error bound, at the time-sliced position of the active unit
            if (w.mode == JFGPU_MODE_MIXED) {
                for (int j = warp; j < 3; j += warps) {
                    double sep[3], p[3];
                    periodic_separation(pa, targets + 3 * j, w.length, sep);
                    permute3(sep, d, p);
                    float value, value_error;
                    mic_x_warp32(w.coulomb, (float)p[0], (float)p[1], (float)p[2], lane, value, value_error);
                    if (lane == 0) {
                        const double scale = w.coulomb.coulomb_prefactor * ca * charge[3 * other + j] * w.speed;
                        pair32[j] = (float)scale * value;
                        error32[j] = fabsf((float)scale) * value_error + fabsf((float)scale * value) * 2.4e-7f;
                        // bounding derivative pp s_x / |s|^3 times the speed: within about 14 ulp, taken as 32
                        const float x = (float)p[0], y = (float)p[1], z = (float)p[2];
                        const float r2 = x * x + y * y + z * z;
                        const float b = (float)(w.coulomb.bound_prefactor * ca * charge[3 * other + j]) * x /
                                        (r2 * sqrtf(r2)) * w.speed32;
                        bound32[j] = b - fabsf(b) * 32.f * 0x1p-24f;  // a lower bound
                    }
                }
                __syncthreads();
            }
            // 0 rejected, 1 thinning in FP64, 2 accepted; every thread takes the same decision
            int decision = 1;
            if (w.mode == JFGPU_MODE_MIXED) {
                // max(0, factor) <= uniform(0, bounding rate) is certain when the factor's upper bound stays below
                // the draw times a lower bound of the bounding rate
                float bounding = 0.f;
                for (int j = 0; j < 3; ++j) bounding += fmaxf(bound32[j], 0.f);
                const double thinning_lower = (double)bounding * draws[0] * (1.0 - 0x1p-20);
                const float factor = pair32[0] + pair32[1] + pair32[2];
                const float error = error32[0] + error32[1] + error32[2] + fabsf(factor) * 2.4e-7f;
                if ((double)factor + (double)error < thinning_lower) decision = 0;  // rejection certain
            }
            if (threadIdx.x == 0) {
                ++s.composite_events;
                if (decision) ++s.thinning_exact;
            }
            if (decision) {
                // the FP64 bounding derivatives (threads 0-2) and merged-image sums (warp j for target unit j)
                if (threadIdx.x < 3) {
                    double sep[3];
                    periodic_separation(pa, targets + 3 * threadIdx.x, w.length, sep);
                    bound[threadIdx.x] =
                        bound_derivative(w.coulomb, d, w.speed, sep, ca, charge[3 * other + threadIdx.x]);
                }
                for (int j = warp; j < 3; j += warps) {
                    double sep[3];
                    periodic_separation(pa, targets + 3 * j, w.length, sep);
                    const double value =
                        coulomb_derivative_warp(w.coulomb, d, w.speed, sep, ca, charge[3 * other + j], lane);
                    if (lane == 0) pair[j] = value;
                }
                __syncthreads();
                double target_factor[3], bounding_rate, event_rate;
                decision = composite_thinning(w.coulomb, JFGPU_DRAW_UNIT, bound, pair, draws, target_factor,
                                              bounding_rate, event_rate) ? 2 : 0;
            }
            if (decision == 2) {
                // the derivatives of the two other local units against the three target units
                for (int k = warp; k < 6; k += warps) {
                    const int i = k / 3 < t ? k / 3 : k / 3 + 1, j = k % 3;
                    double sep[3];
                    periodic_separation(locals + 3 * i, targets + 3 * j, w.length, sep);
                    const double value = coulomb_derivative_warp(w.coulomb, d, w.speed, sep, charge[3 * m + i],
                                                                 charge[3 * other + j], lane);
                    if (lane == 0) cross[i * 3 + j] = value;
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    double target_factor[3], bounding_rate, event_rate, local_cross[9];
                    composite_thinning(w.coulomb, JFGPU_DRAW_UNIT, bound, pair, draws, target_factor, bounding_rate,
                                       event_rate);
                    for (int k = 0; k < 9; ++k) local_cross[k] = cross[k];
                    int new_active = -1;
                    const int lst = composite_lifting(w.coulomb, JFGPU_DRAW_UNIT, t, m < other, event_rate,
                                                      target_factor, local_cross, draws, new_active);
                    if (lst) {
                        s.status = lst;
                    } else {
                        ++s.composite_accepted;
                        s.active = new_active < 3 ? 3 * m + new_active : 3 * other + (new_active - 3);
                    }
                }
            }
            accepted = decision == 2;
        } else if (threadIdx.x == 0) {
            if (best.kind == JFGPU_EV_BOND || best.kind == JFGPU_EV_PAIR) {
                s.active = best.target;
                if (best.kind == JFGPU_EV_BOND) ++s.bond_events; else ++s.lj_events;
            } else if (best.kind == JFGPU_EV_END_OF_CHAIN) {
                s.direction = (s.direction + 1) % 3;
                s.active = best.target;
                // the next end of chain from the time stamp of this event
                time_add(best.q, best.r, time_sub(best.q, best.r, best.q, best.r) + w.chain_time, s.eoc_q, s.eoc_r);
                s.eoc_new_active = water_new_active(w, key, ev + 1);
                ++s.eoc_events;
            } else {
                s.status = JFGPU_STATUS_ASSERTION;
            }
        }
        if (threadIdx.x == 0) {
            for (int c = 0; c < 3; ++c) pos[3 * act + c] = pa[c];
            s.time_q = best.q;
            s.time_r = best.r;
            if (a.log) {
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
            s.refined_items += refined;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) a.state[chain] = s;
}

// ---------------------------------------------------------------------------------------------------------------
// Water with molecular cells
// ---------------------------------------------------------------------------------------------------------------
// int(x / side) along one axis: the exact cell bounds hold cell_min[i] <= x <= cell_max[i] if and only if
// int(x / side) == i, so a multiply by 1 / side guesses the index and a step or two against the bounds corrects it
// The compares with the cell bounds are taken on the bit patterns, which order the non-negative doubles as integers
// (no FP64 compare); x < 0, -0.0, NaN and x >= m side take the division as before.
__device__ inline long long water_axis_index(const WaterCells &cl, double x) {
    const long long bx = (long long)double_bits(x);
    if (bx < 0 || !(x < (double)cl.m * cl.side)) return (long long)(x / cl.side);
    long long i = (long long)(x * cl.inv_side);
    if (i > cl.m - 1) i = cl.m - 1;
    if (i < 0) i = 0;
    while (i > 0 && bx < (long long)double_bits(cl.cell_min[i])) --i;
    while (bx > (long long)double_bits(cl.cell_max[i])) {
        if (i == cl.m - 1) return cl.m;
        ++i;
    }
    return i;
}

// position_to_cell of a root unit (cuboid_cells.py:190-211): int(x / side) along every axis
__device__ inline int water_cell_of(const WaterCells &cl, const double *p, int &cell) {
    const long long ix = water_axis_index(cl, p[0]), iy = water_axis_index(cl, p[1]), iz = water_axis_index(cl, p[2]);
    const long long idx = ix + (long long)cl.m * iy + (long long)cl.m * cl.m * iz;
    if (idx < 0 || idx >= cl.ncells) return JFGPU_STATUS_CELL_RANGE;
    cell = (int)idx;
    return JFGPU_STATUS_OK;
}

__device__ inline void water_cell_axes(const WaterCells &cl, int cell, int *a) {
    a[0] = cell % cl.m;
    a[1] = (cell / cl.m) % cl.m;
    a[2] = cell / (cl.m * cl.m);
}

// SingleActiveCellOccupancy.update (single_active_cell_occupancy.py:149-203) with one occupant per cell: a new
// active molecule returns the previous one to its cell (its occupant when the cell is empty, else a surplus
// molecule of it) and leaves its own cell (as its occupant or as a surplus molecule of it); the same active molecule
// only takes the cell of its root unit again
__device__ inline int water_occupancy_update(const WaterCells &cl, JfgpuWaterCellState &cs, int32_t *occ,
                                             int32_t *sur, const double *roots, int m) {
    if (m != cs.occ_active) {
        if (cs.occ_active >= 0) {
            if (occ[cs.occ_cell] < 0)
                occ[cs.occ_cell] = cs.occ_active;
            else
                sur[cs.occ_active] = cs.occ_cell;
        }
        JF_TRY(water_cell_of(cl, roots + 3 * m, cs.occ_cell));
        cs.occ_active = m;
        if (occ[cs.occ_cell] == m)
            occ[cs.occ_cell] = -1;
        else if (sur[m] == cs.occ_cell)
            sur[m] = -1;
        else
            return JFGPU_STATUS_ASSERTION;  // list.remove of an identifier that is not there
        return JFGPU_STATUS_OK;
    }
    return water_cell_of(cl, roots + 3 * m, cs.occ_cell);
}

__device__ inline void water_no_candidate(WaterCand &c) {
    c.q = INFINITY;
    c.r = INFINITY;
    c.kind = 1 << 30;
    c.target = 1 << 30;
}

// The molecular cell veto of the active molecule in cell `cell` (abstracts/cell_veto_event_handler.py:200-238 with
// the charge factor of DipoleMonteCarloEstimator.charge_correction_factor without target charges: the active unit's
// charge)
__device__ inline int water_veto_candidate(const WaterModel &w, uint64_t key, uint64_t ev, int cell, int d, double ca,
                                           double ts_q, double ts_r, WaterCand &veto, int &veto_cell,
                                           double &veto_rate) {
    const WaterCells &cl = w.cells;
    double charge_factor = ca;
    int which = 0;
    if (!(charge_factor > 0.0)) {
        charge_factor *= -1.0;
        which = 1;
    }
    const WalkerDev &wk = cl.walker[which][d];
    const double total_rate = wk.total_rate * charge_factor;
    const int k = (int)randbelow(draw(key, ev, kRngVetoChoice, 0), (uint32_t)wk.size);
    const double u = wk.mean_rate * uniform53(draw(key, ev, kRngVetoUniform, 0));
    const int rc = (u <= wk.first_rate[k]) ? wk.first_item[k] : wk.second_item[k];
    veto_rate = (which == 0 ? cl.bound_upper[rc * 3 + d] : cl.bound_lower[rc * 3 + d]) * charge_factor;
    if (!(veto_rate > 0.0)) return JFGPU_STATUS_ASSERTION;
    int a[3], b[3];
    water_cell_axes(cl, cell, a);
    water_cell_axes(cl, rc, b);
    veto_cell = cl.tra[a[0] * cl.m + b[0]] + cl.m * cl.tra[a[1] * cl.m + b[1]] +
                cl.m * cl.m * cl.tra[a[2] * cl.m + b[2]];
    const double dt = expovariate(draw(key, ev, kRngVetoTime, 0), w.beta) / (total_rate * w.speed);
    water_no_candidate(veto);
    water_offer(veto, ts_q, ts_r, dt, JFGPU_EV_CELL_VETO, -1);
    return JFGPU_STATUS_OK;
}

// The cell boundary of the active root unit at root in cell `cell` (cell_boundary_event_handler.py:98-156)
__device__ inline void water_boundary_candidate(const WaterModel &w, int cell, int d, const double *root,
                                                double ts_q, double ts_r, WaterCand &bnd, double &boundary) {
    const WaterCells &cl = w.cells;
    int a[3];
    water_cell_axes(cl, cell, a);
    boundary = cl.cell_min[a[d] + 1 == cl.m ? 0 : a[d] + 1];
    double sep = boundary - root[d];
    if (sep < 0.0) sep = sep + w.length;
    water_no_candidate(bnd);
    water_offer(bnd, ts_q, ts_r, sep / cl.root_speed, JFGPU_EV_BOUNDARY, -1);
}

// The molecular cell-bounding factor of the active unit (charge ca, direction d) with molecule `other` in a far
// cell (two_composite_object_cell_bounding_potential_event_handler.py:153-207): the relative cell of the target's root
// cell to the active cell (asserted not nearby), the bound of that cell and direction times the charge factor
// (CellBoundingPotential.standard_velocity_displacement, cell_bounding_potential.py:155-198, with
// DipoleMonteCarloEstimator.charge_correction_factor); rate per unit length, time for the potential change du.
__device__ inline int water_cell_bound(const WaterModel &w, const double *roots, const double *charge, int other,
                                       int active_cell, int d, double ca, double du, double &rate, double &time) {
    const WaterCells &cl = w.cells;
    int target_cell;
    JF_TRY(water_cell_of(cl, roots + 3 * other, target_cell));
    int a[3], b[3];
    water_cell_axes(cl, target_cell, a);
    water_cell_axes(cl, active_cell, b);
    int rc = 0;
    bool near = true;
    for (int k = 2; k >= 0; --k) {
        const int r = cl.rel[a[k] * cl.m + b[k]];
        rc = rc * cl.m + r;
        bool in = false;
        for (int o = 0; o < cl.n_off; ++o) in = in || cl.offsets[o] == r;
        near = near && in;
    }
    if (near) return JFGPU_STATUS_ASSERTION;  // the tagger yields far cells only
    double upper[3], lower[3], velocity[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k) {
        upper[k] = cl.bound_upper[rc * 3 + k];
        lower[k] = -cl.bound_lower[rc * 3 + k];  // stored negated
    }
    velocity[d] = w.speed;
    return composite_cell_bound_time(upper, lower, velocity, ca, charge + 3 * other, 3, cl.dipole_charge, du, rate,
                                     time);
}

__device__ inline void block_reduce_cand(WaterCand &best, WaterCand *warp_slots, int lane, int warp, int warps) {
    for (int offset = 16; offset > 0; offset >>= 1) shuffle_better(best, offset);
    if (lane == 0) warp_slots[warp] = best;
}

// One block of `warps` warps advances one chain of water with molecular cells.  Per event: thread 0 updates the
// occupancy and takes the single candidates (cell veto, cell boundary); the block lists the target molecules (the
// occupants of the nearby cells and the surplus molecules) in shared memory; the candidate items are the three units
// of every target (the summed-bounding Coulomb factor), and, unless the bond and Lennard-Jones candidates are still
// alive from before a cell-boundary event, Lennard-Jones against every other oxygen and the two bonds.  The pair
// items are always solved in FP64 (their earliest is kept for the events after a cell boundary); in the mixed mode
// the Coulomb items are screened in FP32 against the smallest time some candidate surely reaches, and only the
// listed ones are solved in FP64.  The out-state of a Coulomb factor or of a cell veto with a target shares the
// merged-image sums among the warps as the all-pairs kernel does.  The committed active leaf and root unit are
// time-sliced from the in-state of the winner: the current one, or for a bond or Lennard-Jones event the copies its
// candidate took when it was created.
__global__ void __launch_bounds__(256, 2) water_cells_kernel(WaterArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    const int64_t chain = blockIdx.x;
    if (chain >= a.chains) return;  // whole blocks
    const WaterModel &w = a.w;
    const WaterCells &cl = w.cells;
    const int M = w.molecules;
    const uint64_t key = chain_key(w.seed, (uint64_t)(a.first_chain + chain));
    double *pos = a.positions + (size_t)chain * 9 * M;
    double *roots = a.roots + (size_t)chain * 3 * M;
    int32_t *occ = a.occ + (size_t)chain * cl.ncells;
    int32_t *sur = a.sur + (size_t)chain * M;
    const double *charge = a.charges;
    __shared__ JfgpuWaterState s;
    __shared__ JfgpuWaterCellState cs;
    __shared__ WaterCand warp_best[kMaxWarps], warp_pair[kMaxWarps];
    __shared__ float warp_upper[kMaxWarps], warp_pair_upper[kMaxWarps];
    extern __shared__ float dynamic[];
    const int items_cap = water_cells_items_max(M);
    float *lower = dynamic;
    int *list = reinterpret_cast<int *>(dynamic + items_cap);
    int *chunk_count = list + items_cap;
    int *targets = chunk_count + ((items_cap + 31) >> 5);
    int *far_targets = targets + 4 * M;  // after the screen's prefactors [3 M]
    __shared__ int status, single_status, n_targets, n_far, veto_cell, pp_active;
    __shared__ float veto_bound, other_bound;
    __shared__ WaterCand veto, bnd;
    float *pp32 = reinterpret_cast<float *>(targets + M);  // [3 M]
    __shared__ double veto_rate, boundary;
    __shared__ double bound[3], pair[3], cross[9];
    __shared__ float pair32[3], error32[3];
    if (threadIdx.x == 0) {
        s = a.state[chain];
        cs = a.cell_state[chain];
        s.stopped = 0;
        status = JFGPU_STATUS_OK;
        single_status = JFGPU_STATUS_OK;
        pp_active = -1;
    }
    __syncthreads();
    for (int64_t step = 0; step < a.events && s.status == JFGPU_STATUS_OK; ++step) {
        const int act = s.active, m = act / 3, t = act % 3, d = s.direction;
        const uint64_t ev = (uint64_t)s.events;
        const double ts_q = s.time_q, ts_r = s.time_r;
        const double ca = charge[act];
        // the occupancy (thread 0) and, beside it, the single candidates from the cell of the active root unit
        // (the first thread of the second warp, or thread 0 of a one-warp block)
        if (threadIdx.x == 0) {
            n_targets = 0;
            n_far = 0;
            status = water_occupancy_update(cl, cs, occ, sur, roots, m);
        }
        // the cell veto (the first thread of the second warp) and the cell boundary with the bounds of the end of
        // chain and of a kept pair candidate (the first thread of the third warp), each from the cell of the active
        // root unit, beside the occupancy update; with fewer warps the same threads take more of them
        const int veto_thread = warps > 1 ? 32 : 0, boundary_thread = warps > 2 ? 64 : veto_thread;
        if (threadIdx.x == veto_thread) {
            int cell;
            int st = water_cell_of(cl, roots + 3 * m, cell);
            if (cl.far == JFGPU_FAR_CELL_VETO) {
                if (!st) st = water_veto_candidate(w, key, ev, cell, d, ca, ts_q, ts_r, veto, veto_cell, veto_rate);
            } else {
                water_no_candidate(veto);  // the cell-bounding factors are items of the block's screen
            }
            veto_bound = __double2float_ru(time_sub(veto.q, veto.r, ts_q, ts_r));
            single_status = st;
        }
        if (threadIdx.x == boundary_thread) {
            // the time since the time stamp that these candidates surely reach, rounded up (the screen's bound)
            int cell;
            if (water_cell_of(cl, roots + 3 * m, cell) == JFGPU_STATUS_OK) {
                water_boundary_candidate(w, cell, d, roots + 3 * m, ts_q, ts_r, bnd, boundary);
            } else {
                water_no_candidate(bnd);  // the veto thread reports the cell error
            }
            float sb = __double2float_ru(time_sub(bnd.q, bnd.r, ts_q, ts_r));
            sb = fminf(sb, __double2float_ru(time_sub(s.eoc_q, s.eoc_r, ts_q, ts_r)));
            if (cs.pairs_valid) sb = fminf(sb, __double2float_ru(time_sub(cs.pair_q, cs.pair_r, ts_q, ts_r)));
            other_bound = sb;
        }
        if (act != pp_active) {
            // the FP32 prefactors of the Coulomb screen for a new active unit
            for (int b = threadIdx.x; b < 3 * M; b += blockDim.x)
                pp32[b] = (float)(w.coulomb.bound_prefactor * ca * charge[b]);
        }
        __syncthreads();
        if (threadIdx.x == 0) pp_active = act;
        const WaterCand single = water_better(bnd, veto) ? bnd : veto;
        const float single_bound = fminf(veto_bound, other_bound);
        if (status != JFGPU_STATUS_OK || single_status != JFGPU_STATUS_OK) {
            if (threadIdx.x == 0) s.status = status != JFGPU_STATUS_OK ? status : single_status;
            break;
        }
        // the target molecules: the occupants of the nearby cells (ExcludedCellsTagger), the surplus molecules
        {
            int ax[3];
            water_cell_axes(cl, cs.occ_cell, ax);
            const int n_near = cl.n_off * cl.n_off * cl.n_off;
            for (int k = threadIdx.x; k < n_near + M; k += blockDim.x) {
                int other = -1;
                if (k < n_near) {
                    const int ox = k % cl.n_off, oy = (k / cl.n_off) % cl.n_off, oz = k / (cl.n_off * cl.n_off);
                    const int cell = (ax[0] + cl.offsets[ox]) % cl.m + cl.m * ((ax[1] + cl.offsets[oy]) % cl.m) +
                                     cl.m * cl.m * ((ax[2] + cl.offsets[oz]) % cl.m);
                    other = occ[cell];
                } else if (sur[k - n_near] >= 0) {
                    other = k - n_near;
                }
                if (other >= 0) targets[atomicAdd(&n_targets, 1)] = other;
            }
            if (cl.far == JFGPU_FAR_CELL_BOUNDING) {
                // CellBoundingPotentialTagger: the occupant of every occupied cell that is not nearby
                for (int k = threadIdx.x; k < cl.ncells; k += blockDim.x) {
                    const int other = occ[k];
                    if (other < 0) continue;
                    int c[3];
                    water_cell_axes(cl, k, c);
                    bool near = true;
                    for (int axis = 0; axis < 3; ++axis) {
                        const int r = (c[axis] - ax[axis] + cl.m) % cl.m;
                        bool in = false;
                        for (int o = 0; o < cl.n_off; ++o) in = in || cl.offsets[o] == r;
                        near = near && in;
                    }
                    if (!near) far_targets[atomicAdd(&n_far, 1)] = other;
                }
            }
        }
        __syncthreads();
        const int nt = n_targets, nf = n_far;
        const bool new_pairs = !cs.pairs_valid;
        double pa[3], pr[3], pa0[3], pr0[3];
        for (int c = 0; c < 3; ++c) {
            pa[c] = pa0[c] = pos[3 * act + c];
            pr[c] = pr0[c] = roots[3 * m + c];
        }
        WaterCand eoc;
        eoc.q = s.eoc_q;
        eoc.r = s.eoc_r;
        eoc.kind = JFGPU_EV_END_OF_CHAIN;
        eoc.target = s.eoc_new_active;
        WaterCand best, pbest;
        best.q = pbest.q = INFINITY;
        best.r = pbest.r = INFINITY;
        best.kind = pbest.kind = 1 << 30;
        best.target = pbest.target = 1 << 30;
        // items: the Coulomb factors' units by unit type, the far cell-bounding factors, the pair items
        const int group = (nt + 31) & ~31, n_near_items = 3 * group;
        const int n_coulomb = n_near_items + ((nf + 31) & ~31);
        const int n_lj = new_pairs && t == 1 ? M - 1 : 0, n_pairs = new_pairs ? n_lj + 2 : 0;
        const int items = n_coulomb + n_pairs;
        const bool mixed = w.mode == JFGPU_MODE_MIXED;
        int st = JFGPU_STATUS_OK, refined = nt * 3 + nf + n_pairs;
        // phase A: the pair items in FP64; the Coulomb items in FP64 (exact mode) or screened in FP32 (mixed mode:
        // lower[item] = the earliest time the item may reach, -inf where the screen cannot decide)
        float mine = INFINITY, pair_mine = INFINITY;
        for (int item = threadIdx.x; item < items && !st; item += blockDim.x) {
            if (item >= n_coulomb) {
                const int k = item - n_coulomb;
                if (mixed) {
                    // Lennard-Jones screened in FP32 (a lower and an upper bound), a bond bounded from below
                    float t32, e32 = 0.f;
                    bool unsafe = false;
                    if (k < n_lj)
                        lj_unit_screen(w, pos, key, ev, k + (k >= m), d, pa, t32, e32, unsafe);
                    else
                        bond_unit_screen(w, pos, key, ev, m, t, k - n_lj, pa, t32, unsafe);
                    lower[item] = unsafe ? -INFINITY : __fsub_rd(t32, e32);
                    if (!unsafe && k < n_lj) pair_mine = fminf(pair_mine, __fadd_ru(t32, e32));
                    continue;
                }
                st = pair_item_exact(w, pos, key, ev, k, n_lj, m, t, d, pa, ts_q, ts_r, pbest);
                continue;
            }
            if (item >= n_near_items) {
                // a far cell-bounding factor: its bound times the charge factor, the potential change keyed by the
                // target molecule; screened in FP32 with the potential change's FP32 error (24 units of 2^-24) and
                // the roundings of the rate and the division, taken as 64 units
                const int f = item - n_near_items;
                if (f >= nf) {
                    lower[item] = INFINITY;  // padding
                    continue;
                }
                const int other = far_targets[f];
                const uint64_t bits = draw(key, ev, kRngCellBound, (uint32_t)other);
                if (mixed) {
                    const uint64_t n = bits >> 11;
                    const float du32 = n < (1ull << 52) ? -log1pf(-(float)n * 0x1p-53f) / w.beta32
                                                        : -logf((float)((1ull << 53) - n) * 0x1p-53f) / w.beta32;
                    double rate, time;
                    st = water_cell_bound(w, roots, charge, other, cs.occ_cell, d, ca, 1.0, rate, time);
                    if (st) continue;
                    const float t32 = rate > 0.0 ? du32 / (float)rate / w.speed32 : INFINITY;
                    lower[item] = t32 * (1.f - 64.f * 0x1p-24f);
                    mine = fminf(mine, t32 * (1.f + 64.f * 0x1p-24f));
                } else {
                    double rate, time;
                    st = water_cell_bound(w, roots, charge, other, cs.occ_cell, d, ca, expovariate(bits, w.beta),
                                          rate, time);
                    if (!st) water_offer(best, ts_q, ts_r, time, JFGPU_EV_CELL_BOUNDING, other);
                }
                continue;
            }
            const int j = item / group, k = item % group;
            if (k >= nt) {
                lower[item] = INFINITY;  // padding
                continue;
            }
            if (mixed) {
                float t32, e32;
                bool unsafe = false;
                coulomb_unit_screen(w, pos, charge, key, ev, targets[k], j, d, pa, ca, t32, e32, unsafe, pp32);
                lower[item] = unsafe ? -INFINITY : __fsub_rd(t32, e32);
                if (!unsafe) mine = fminf(mine, __fadd_ru(t32, e32));
            } else {
                coulomb_unit_exact(w, pos, charge, key, ev, targets[k], j, d, pa, ca, ts_q, ts_r, best);
            }
        }
        if (st) status = st;  // any failing thread; all stop after the barrier
        block_reduce_cand(pbest, warp_pair, lane, warp, warps);
        if (mixed) {
            for (int offset = 16; offset > 0; offset >>= 1) {
                mine = fminf(mine, __shfl_xor_sync(kFull, mine, offset));
                pair_mine = fminf(pair_mine, __shfl_xor_sync(kFull, pair_mine, offset));
            }
            if (lane == 0) {
                warp_upper[warp] = mine;
                warp_pair_upper[warp] = pair_mine;
            }
        }
        __syncthreads();
        if (status != JFGPU_STATUS_OK) {
            if (threadIdx.x == 0) s.status = status;
            break;
        }
        pbest = warp_pair[0];
        for (int k = 1; k < warps; ++k)
            if (water_better(warp_pair[k], pbest)) pbest = warp_pair[k];
        WaterCand pcand = pbest;
        if (!new_pairs) {
            pcand.q = cs.pair_q;
            pcand.r = cs.pair_r;
            pcand.kind = cs.pair_kind;
            pcand.target = cs.pair_target;
        }
        if (mixed) {
            // the bound: the smallest time that some candidate surely reaches (a screened Coulomb or Lennard-Jones
            // time plus its error bound, the pair candidate kept across a cell boundary, the single candidates, the
            // end of chain), in time since the time stamp, rounded up
            float bound_time = single_bound;
            for (int k = 0; k < warps; ++k) bound_time = fminf(bound_time, fminf(warp_upper[k], warp_pair_upper[k]));
            // the items that may come first, listed in item order (the Coulomb items by unit type, so that a warp of
            // the FP64 pass follows one charge sign; then the pair items): the taken count of every chunk of 32
            // items, then every warp writes the items of its chunks at their offsets
            const int chunks = (items + 31) >> 5;
            for (int c = warp; c < chunks; c += warps) {
                const int item = 32 * c + lane;
                const unsigned votes = __ballot_sync(kFull, item < items && lower[item] <= bound_time);
                if (lane == 0) chunk_count[c] = __popc(votes);
            }
            __syncthreads();
            int taken = 0;
            for (int c = 0; c < chunks; ++c) {
                if (c % warps == warp) {
                    const int item = 32 * c + lane;
                    const bool take = item < items && lower[item] <= bound_time;
                    const unsigned votes = __ballot_sync(kFull, take);
                    if (take) list[taken + __popc(votes & ((1u << lane) - 1u))] = item;
                }
                taken += chunk_count[c];
            }
            __syncthreads();
            // phase B: the FP64 solve of the listed items
            for (int v = threadIdx.x; v < taken && !st; v += blockDim.x) {
                const int item = list[v];
                if (item >= n_coulomb) {
                    st = pair_item_exact(w, pos, key, ev, item - n_coulomb, n_lj, m, t, d, pa, ts_q, ts_r, pbest);
                    continue;
                }
                if (item >= n_near_items) {
                    const int f = item - n_near_items;
                    if (f >= nf) continue;  // padding
                    const int other = far_targets[f];
                    double rate, time;
                    st = water_cell_bound(w, roots, charge, other, cs.occ_cell, d, ca,
                                          expovariate(draw(key, ev, kRngCellBound, (uint32_t)other), w.beta), rate,
                                          time);
                    if (!st) water_offer(best, ts_q, ts_r, time, JFGPU_EV_CELL_BOUNDING, other);
                    continue;
                }
                if (item % group >= nt) continue;  // padding (listed only under an infinite bound)
                coulomb_unit_exact(w, pos, charge, key, ev, targets[item % group], item / group, d, pa, ca, ts_q,
                                   ts_r, best);
            }
            if (st) status = st;
            refined = taken;
            if (new_pairs) {
                // the earliest of the listed pair items: the winner when a pair item comes first
                block_reduce_cand(pbest, warp_pair, lane, warp, warps);
                __syncthreads();
                if (status != JFGPU_STATUS_OK) {
                    if (threadIdx.x == 0) s.status = status;
                    break;
                }
                pbest = warp_pair[0];
                for (int k = 1; k < warps; ++k)
                    if (water_better(warp_pair[k], pbest)) pbest = warp_pair[k];
                pcand = pbest;
            }
        }
        block_reduce_cand(best, warp_best, lane, warp, warps);
        __syncthreads();
        // every thread takes the winner: the warps' best, the pair candidate, the single candidates, the end of
        // chain, the stop time (which wins ties)
        best = warp_best[0];
        for (int k = 1; k < warps; ++k)
            if (water_better(warp_best[k], best)) best = warp_best[k];
        if (water_better(pcand, best)) best = pcand;
        if (water_better(single, best)) best = single;
        if (water_better(eoc, best)) best = eoc;
        if (mixed && new_pairs && best.kind == JFGPU_EV_BOUNDARY && cl.keep_pairs) {
            // the pair candidates outlive a cell boundary: the earliest of all of them in FP64 (the screen listed only
            // those that could come first at this event)
            WaterCand all;
            all.q = INFINITY;
            all.r = INFINITY;
            all.kind = 1 << 30;
            all.target = 1 << 30;
            for (int k = threadIdx.x; k < n_pairs && !st; k += blockDim.x)
                st = pair_item_exact(w, pos, key, ev, k, n_lj, m, t, d, pa, ts_q, ts_r, all);
            if (st) status = st;
            block_reduce_cand(all, warp_pair, lane, warp, warps);
            __syncthreads();
            if (status != JFGPU_STATUS_OK) {
                if (threadIdx.x == 0) s.status = status;
                break;
            }
            pbest = warp_pair[0];
            for (int k = 1; k < warps; ++k)
                if (water_better(warp_pair[k], pbest)) pbest = warp_pair[k];
            refined += n_pairs;
        }
        if (!isinf(a.stop_q) && !time_lt(best.q, best.r, a.stop_q, a.stop_r)) {
            // the end of the run: the active leaf and root unit time-sliced to the stop time, no event; the pair
            // candidates are created anew by the next call
            if (threadIdx.x == 0) {
                const double dt = time_sub(a.stop_q, a.stop_r, ts_q, ts_r);
                for (int c = 0; c < 3; ++c) {
                    pos[3 * act + c] = py_mod_near(pa[c] + (c == d ? w.speed : 0.0) * dt, w.length);
                    roots[3 * m + c] = py_mod_near(pr[c] + (c == d ? cl.root_speed : 0.0) * dt, w.length);
                }
                s.time_q = a.stop_q;
                s.time_r = a.stop_r;
                s.stopped = 1;
                cs.pairs_valid = 0;
            }
            break;
        }
        // commit: the active leaf and root unit time-sliced from the winner's in-state
        {
            const bool stale = (best.kind == JFGPU_EV_BOND || best.kind == JFGPU_EV_PAIR) && !new_pairs;
            const double from_q = stale ? cs.snap_q : ts_q, from_r = stale ? cs.snap_r : ts_r;
            const double dt = time_sub(best.q, best.r, from_q, from_r);
            for (int c = 0; c < 3; ++c) {
                const double leaf = stale ? cs.snap_leaf[c] : pa0[c], root = stale ? cs.snap_root[c] : pr0[c];
                pa[c] = py_mod_near(leaf + (c == d ? w.speed : 0.0) * dt, w.length);
                pr[c] = py_mod_near(root + (c == d ? cl.root_speed : 0.0) * dt, w.length);
            }
        }
        int accepted = 1;
        int other = -1;
        double given_rate = veto_rate;
        if (best.kind == JFGPU_EV_COMPOSITE) other = best.target;
        if (best.kind == JFGPU_EV_CELL_VETO) {
            other = occ[veto_cell];  // the occupant of the sampled cell (Mediator.get_arguments_cell_veto_event_handler)
            accepted = 0;
        }
        if (best.kind == JFGPU_EV_CELL_BOUNDING) {
            // send_out_state (:209-265): the active root is still in the candidate's cell (the reference has no
            // out-state otherwise), and the thinning draws against the bounding event rate times the speed
            other = best.target;
            int now_cell;
            double rate, time;
            int cst = water_cell_of(cl, pr, now_cell);
            if (!cst && now_cell != cs.occ_cell) cst = JFGPU_STATUS_ASSERTION;
            if (!cst) cst = water_cell_bound(w, roots, charge, other, cs.occ_cell, d, ca, 1.0, rate, time);
            if (cst) {
                if (threadIdx.x == 0) s.status = cst;
                other = -1;
            }
            given_rate = rate * w.speed;
        }
        if (other >= 0) {
            const bool veto = best.kind == JFGPU_EV_CELL_VETO || best.kind == JFGPU_EV_CELL_BOUNDING;
            const double *locals = pos + 9 * m, *targets_pos = pos + 9 * other;
            double draws[3];
            draws[0] = uniform53(draw(key, ev, kRngThin, 0));
            draws[1] = uniform53(draw(key, ev, kRngLift, 0));
            draws[2] = draws[1];
            if (mixed) {
                for (int j = warp; j < 3; j += warps) {
                    double sep[3], p[3];
                    periodic_separation(pa, targets_pos + 3 * j, w.length, sep);
                    permute3(sep, d, p);
                    float value, value_error;
                    mic_x_warp32(w.coulomb, (float)p[0], (float)p[1], (float)p[2], lane, value, value_error);
                    if (lane == 0) {
                        const double scale = w.coulomb.coulomb_prefactor * ca * charge[3 * other + j] * w.speed;
                        pair32[j] = (float)scale * value;
                        error32[j] = fabsf((float)scale) * value_error + fabsf((float)scale * value) * 2.4e-7f;
                        // the summed bound of a Coulomb factor: its bounding derivative pp s_x / |s|^3 times the
                        // speed, within about 14 ulp, taken as 32 (a lower bound)
                        const float x = (float)p[0], y = (float)p[1], z = (float)p[2];
                        const float r2 = x * x + y * y + z * z;
                        const float b = (float)(w.coulomb.bound_prefactor * ca * charge[3 * other + j]) * x /
                                        (r2 * sqrtf(r2)) * w.speed32;
                        bound[j] = (double)(b - fabsf(b) * 32.f * 0x1p-24f);
                    }
                }
                __syncthreads();
            }
            // 0 rejected, 1 thinning in FP64, 2 accepted; every thread takes the same decision
            int decision = 1;
            if (mixed) {
                // max(0, factor) <= uniform(0, bounding rate) is certain when the factor's upper bound stays below
                // the draw times a lower bound of the bounding rate
                double bounding = given_rate;
                if (!veto) {
                    float sum = 0.f;
                    for (int j = 0; j < 3; ++j) sum += fmaxf((float)bound[j], 0.f);
                    bounding = (double)sum;
                }
                const double thinning_lower = bounding * draws[0] * (1.0 - 0x1p-20);
                const float factor = pair32[0] + pair32[1] + pair32[2];
                const float error = error32[0] + error32[1] + error32[2] + fabsf(factor) * 2.4e-7f;
                if ((double)factor + (double)error < thinning_lower) decision = 0;  // rejection certain
                __syncthreads();  // every thread has read the FP32 sums before bound[] is refilled
            }
            if (threadIdx.x == 0) {
                if (!veto) ++s.composite_events;
                if (decision) ++s.thinning_exact;
            }
            if (decision) {
                if (!veto && threadIdx.x < 3) {
                    double sep[3];
                    periodic_separation(pa, targets_pos + 3 * threadIdx.x, w.length, sep);
                    bound[threadIdx.x] =
                        bound_derivative(w.coulomb, d, w.speed, sep, ca, charge[3 * other + threadIdx.x]);
                }
                for (int j = warp; j < 3; j += warps) {
                    double sep[3];
                    periodic_separation(pa, targets_pos + 3 * j, w.length, sep);
                    const double value =
                        coulomb_derivative_warp(w.coulomb, d, w.speed, sep, ca, charge[3 * other + j], lane);
                    if (lane == 0) pair[j] = value;
                }
                __syncthreads();
                double target_factor[3], bounding_rate, event_rate;
                bool confirmed = false;
                if (veto) {
                    if (composite_given_thinning(w.coulomb, JFGPU_DRAW_UNIT, given_rate, pair, draws, target_factor,
                                                 bounding_rate, event_rate, confirmed))
                        confirmed = false;  // the rate was checked when the candidate was made
                } else {
                    confirmed = composite_thinning(w.coulomb, JFGPU_DRAW_UNIT, bound, pair, draws, target_factor,
                                                   bounding_rate, event_rate);
                }
                decision = confirmed ? 2 : 0;
            }
            if (decision == 2) {
                // the derivatives of the two other local units against the three target units
                for (int k = warp; k < 6; k += warps) {
                    const int i = k / 3 < t ? k / 3 : k / 3 + 1, j = k % 3;
                    double sep[3];
                    periodic_separation(locals + 3 * i, targets_pos + 3 * j, w.length, sep);
                    const double value = coulomb_derivative_warp(w.coulomb, d, w.speed, sep, charge[3 * m + i],
                                                                 charge[3 * other + j], lane);
                    if (lane == 0) cross[i * 3 + j] = value;
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    double target_factor[3], bounding_rate, event_rate, local_cross[9];
                    bool confirmed = true;
                    if (veto)
                        composite_given_thinning(w.coulomb, JFGPU_DRAW_UNIT, given_rate, pair, draws, target_factor,
                                                 bounding_rate, event_rate, confirmed);
                    else
                        composite_thinning(w.coulomb, JFGPU_DRAW_UNIT, bound, pair, draws, target_factor,
                                           bounding_rate, event_rate);
                    for (int k = 0; k < 9; ++k) local_cross[k] = cross[k];
                    int new_active = -1;
                    const int lst = composite_lifting(w.coulomb, JFGPU_DRAW_UNIT, t, m < other, event_rate,
                                                      target_factor, local_cross, draws, new_active);
                    if (lst) {
                        s.status = lst;
                    } else {
                        ++s.composite_accepted;
                        s.active = new_active < 3 ? 3 * m + new_active : 3 * other + (new_active - 3);
                    }
                }
            }
            accepted = decision == 2;
        } else if (threadIdx.x == 0) {
            if (best.kind == JFGPU_EV_BOND || best.kind == JFGPU_EV_PAIR) {
                s.active = best.target;
                if (best.kind == JFGPU_EV_BOND) ++s.bond_events; else ++s.lj_events;
            } else if (best.kind == JFGPU_EV_END_OF_CHAIN) {
                s.direction = (s.direction + 1) % 3;
                s.active = best.target;
                time_add(best.q, best.r, time_sub(best.q, best.r, best.q, best.r) + w.chain_time, s.eoc_q, s.eoc_r);
                s.eoc_new_active = water_new_active(w, key, ev + 1);
                ++s.eoc_events;
            } else if (best.kind == JFGPU_EV_BOUNDARY) {
                accepted = 0;
                ++cs.boundary_events;
            } else if (best.kind != JFGPU_EV_CELL_VETO && best.kind != JFGPU_EV_CELL_BOUNDING) {
                s.status = JFGPU_STATUS_ASSERTION;
            }
        }
        if (threadIdx.x == 0) {
            if (best.kind == JFGPU_EV_BOUNDARY) pr[d] = boundary;
            if (best.kind == JFGPU_EV_CELL_VETO || best.kind == JFGPU_EV_CELL_BOUNDING) {
                ++cs.veto_events;
                if (other >= 0) ++cs.veto_targets;
            }
            if (new_pairs) {
                // the pair candidates created with this event and the in-state copies they hold
                cs.pair_q = pbest.q;
                cs.pair_r = pbest.r;
                cs.pair_kind = pbest.kind;
                cs.pair_target = pbest.target;
                for (int c = 0; c < 3; ++c) {
                    cs.snap_leaf[c] = pa0[c];
                    cs.snap_root[c] = pr0[c];
                }
                cs.snap_q = ts_q;
                cs.snap_r = ts_r;
            }
            // the cell boundary trashes only the cell-based factors; every other event the pair candidates too
            cs.pairs_valid = best.kind == JFGPU_EV_BOUNDARY && cl.keep_pairs;
            for (int c = 0; c < 3; ++c) {
                pos[3 * act + c] = pa[c];
                roots[3 * m + c] = pr[c];
            }
            s.time_q = best.q;
            s.time_r = best.r;
            if (a.log) {
                JfgpuEvent e;
                e.kind = best.kind;
                e.moved = act;
                e.target = best.kind == JFGPU_EV_CELL_VETO ? other : (best.kind == JFGPU_EV_BOUNDARY ? -1 : best.target);
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
            if (a.root_log)
                for (int c = 0; c < 3; ++c) a.root_log[(chain * a.events + step) * 3 + c] = pr[c];
            ++s.events;
            s.refined_items += refined;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.state[chain] = s;
        a.cell_state[chain] = cs;
    }
}

// the occupancy from the roots (SingleActiveCellOccupancy.initialize, single_active_cell_occupancy.py:95-121: the
// root nodes in order, the first molecule of a cell its occupant, the others surplus), a fresh cell state
__global__ void water_cells_init_kernel(WaterModel w, JfgpuWaterCellBuffers b, int64_t chains) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= chains) return;
    const WaterCells &cl = w.cells;
    const int M = w.molecules;
    int32_t *occ = b.occupancy + (size_t)c * cl.ncells;
    int32_t *sur = b.surplus + (size_t)c * M;
    const double *roots = b.roots + (size_t)c * 3 * M;
    JfgpuWaterCellState cs;
    memset(&cs, 0, sizeof(cs));
    cs.pair_q = cs.pair_r = INFINITY;
    cs.pair_kind = cs.pair_target = 1 << 30;
    cs.occ_active = -1;
    cs.occ_cell = -1;
    for (int k = 0; k < cl.ncells; ++k) occ[k] = -1;
    for (int i = 0; i < M; ++i) {
        sur[i] = -1;
        int cell;
        if (water_cell_of(cl, roots + 3 * i, cell)) {
            cs.reserved = JFGPU_STATUS_CELL_RANGE;
            continue;
        }
        if (occ[cell] < 0)
            occ[cell] = i;
        else
            sur[i] = cell;
    }
    b.cell_state[c] = cs;
}

struct WaterHandle {
    WaterModel model;
    double *fourier = nullptr;
    float *fourier32 = nullptr;
    int4 *terms = nullptr;  // real-space images, then Fourier rows
    int device = -1;
    std::vector<void *> cell_tables;  // device tables of the molecular cells
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
        desc->fourier_cutoff < 0 || desc->position_cutoff < 0 || !(desc->alpha > 0.0) ||
        (desc->mode != JFGPU_MODE_EXACT && desc->mode != JFGPU_MODE_MIXED))
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
    std::vector<float> table32(table.begin(), table.end());
    if (cudaMalloc((void **)&h->fourier32, table32.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(h->fourier32, table32.data(), table32.size() * sizeof(float), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
        if (h->fourier32) cudaFree(h->fourier32);
        cudaFree(h->fourier);
        delete h;
        return JFGPU_ERROR_ALLOCATION;
    }
    std::vector<int4> images, rows;
    merged_image_terms(desc->fourier_cutoff, desc->position_cutoff, images, rows);
    std::vector<int4> terms(images);
    terms.insert(terms.end(), rows.begin(), rows.end());
    if (cudaMalloc((void **)&h->terms, terms.size() * sizeof(int4)) != cudaSuccess) {
        cudaFree(h->fourier32);
        cudaFree(h->fourier);
        delete h;
        return JFGPU_ERROR_ALLOCATION;
    }
    if (cudaMemcpy(h->terms, terms.data(), terms.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(h->terms);
        cudaFree(h->fourier32);
        cudaFree(h->fourier);
        delete h;
        return JFGPU_ERROR_CUDA;
    }
    WaterModel &w = h->model;
    w.coulomb.mic = make_mic(desc->fourier_cutoff, desc->position_cutoff, desc->alpha, desc->system_length,
                             h->fourier);
    w.coulomb.images = h->terms;
    w.coulomb.n_images = (int)images.size();
    w.coulomb.rows = h->terms + images.size();
    w.coulomb.n_rows = (int)rows.size();
    const MIC &mic = w.coulomb.mic;
    w.coulomb.fourier32 = h->fourier32;
    w.coulomb.alpha_over_length32 = (float)mic.alpha_over_length;
    w.coulomb.alpha_over_length_sq32 = (float)mic.alpha_over_length_sq;
    w.coulomb.two_alpha_over_length_root_pi32 = (float)mic.two_alpha_over_length_root_pi;
    w.coulomb.system_length32 = (float)mic.system_length;
    w.coulomb.two_pi_over_length32 = (float)mic.two_pi_over_length;
    w.mode = desc->mode;
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
    w.beta32 = (float)desc->beta;
    w.speed32 = (float)desc->speed;
    w.length32 = (float)desc->system_length;
    w.lj32.a12 = (float)w.lj.twelve.prefactor;
    w.lj32.a6 = (float)w.lj.six.prefactor;
    w.lj32.four_over_k = (float)(4.0 / w.lj.prefactor);
    w.lj32.sigma_sq = (float)(w.lj.sigma * w.lj.sigma);
    w.lj32.r0_sq = (float)w.lj.r0_squared;
    w.margin32 = (float)(16.0 * desc->system_length / 16777216.0);
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
    for (void *p : h->cell_tables) cudaFree(p);
    if (h->fourier) cudaFree(h->fourier);
    if (h->fourier32) cudaFree(h->fourier32);
    if (h->terms) cudaFree(h->terms);
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
                               int64_t chains, int64_t first_chain, int64_t events, double stop_q, double stop_r,
                               JfgpuEvent *log, int32_t warps_per_block, void *stream) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h || chains < 0 || first_chain < 0 || events < 0 || warps_per_block < 0 || warps_per_block > 8)
        return JFGPU_ERROR_ARGUMENT;
    if (chains == 0 || events == 0) return JFGPU_OK;
    if (!positions || !charges || !state) return JFGPU_ERROR_ARGUMENT;
    const int warps = warps_per_block ? warps_per_block : 3;
    WaterArgs a;
    memset(&a, 0, sizeof(a));
    a.w = h->model;
    a.positions = positions;
    a.charges = charges;
    a.state = state;
    a.log = log;
    a.chains = chains;
    a.first_chain = first_chain;
    a.events = events;
    a.stop_q = stop_q;
    a.stop_r = stop_r;
    const size_t shared = water_shared_bytes(h->model.molecules);
    if (shared > 48 * 1024 &&
        cudaFuncSetAttribute(water_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared) != cudaSuccess)
        return JFGPU_ERROR_CUDA;
    water_kernel<<<(unsigned)chains, 32 * warps, shared, static_cast<cudaStream_t>(stream)>>>(a);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

namespace {

template <typename T>
const T *water_table(WaterHandle *h, const std::vector<T> &host, int &error) {
    void *ptr = nullptr;
    const size_t bytes = sizeof(T) * (host.empty() ? 1 : host.size());
    if (cudaMalloc(&ptr, bytes) != cudaSuccess) {
        error = JFGPU_ERROR_ALLOCATION;
        return nullptr;
    }
    h->cell_tables.push_back(ptr);
    if (!host.empty() && cudaMemcpy(ptr, host.data(), sizeof(T) * host.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        error = JFGPU_ERROR_CUDA;
    return static_cast<const T *>(ptr);
}

}  // namespace

extern "C" int jfgpu_water_set_cells(void *water, int32_t cells_per_side, int32_t neighbor_layers,
                                     const double *bounds_upper, const double *bounds_lower, int32_t keep_pairs,
                                     int32_t far, double dipole_charge) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h || cells_per_side < 1 || cells_per_side > 32 || neighbor_layers < 0 || !bounds_upper || !bounds_lower ||
        (far != JFGPU_FAR_CELL_VETO && far != JFGPU_FAR_CELL_BOUNDING) || !(dipole_charge != 0.0))
        return JFGPU_ERROR_ARGUMENT;
    WaterModel &w = h->model;
    WaterCells cl;
    memset(&cl, 0, sizeof(cl));
    const int m = cells_per_side;
    cl.m = m;
    cl.ncells = m * m * m;
    cl.keep_pairs = keep_pairs ? 1 : 0;
    cl.far = far;
    cl.dipole_charge = dipole_charge;
    cl.side = w.length / m;
    cl.inv_side = 1.0 / cl.side;
    cl.root_speed = w.speed * (1.0 / 3.0);  // the leaf velocity times its weight 1 / len(children) in the molecule
    // the residues of the neighbour-layer offsets (cuboid_periodic_cells.py:74-100), ascending
    std::vector<char> near(m, 0);
    for (int o = -neighbor_layers; o <= neighbor_layers; ++o) near[((o % m) + m) % m] = 1;
    for (int r = 0; r < m; ++r)
        if (near[r]) cl.offsets[cl.n_off++] = r;
    std::vector<double> lo, hi;
    cell_bounds(w.length, m, lo, hi);
    // relative_cell / translate along one axis (cuboid_periodic_cells.py:156-207)
    std::vector<int16_t> tra((size_t)m * m), rel((size_t)m * m);
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b) {
            const double center = (hi[a] + lo[a]) / 2.0;
            tra[(size_t)a * m + b] = (int16_t)(long long)(py_mod(center + lo[b], w.length) / cl.side);
            rel[(size_t)a * m + b] = (int16_t)(long long)(py_mod(center - lo[b], w.length) / cl.side);
        }
    auto nearby_zero = [&](int cell) {
        return near[cell % m] && near[(cell / m) % m] && near[cell / (m * m)];
    };
    std::vector<double> upper(bounds_upper, bounds_upper + 3 * (size_t)cl.ncells);
    std::vector<double> lower(bounds_lower, bounds_lower + 3 * (size_t)cl.ncells);
    int error = JFGPU_OK;
    HostWalker walkers[2][3];
    for (int which = 0; which < 2; ++which)
        for (int d = 0; d < 3; ++d) {
            // the cells that are not nearby the zero cell, in the order of yield_cells, with max(bound, 0.0)
            // (cell_veto_event_handler.py:149-160)
            std::vector<int> items;
            std::vector<double> rates;
            for (int cell = 0; cell < cl.ncells; ++cell) {
                if (nearby_zero(cell)) continue;
                const double r = (which == 0 ? upper : lower)[3 * (size_t)cell + d];
                if (std::isnan(r)) return JFGPU_ERROR_TABLE;  // a far cell without a bound
                items.push_back(cell);
                rates.push_back(r > 0.0 ? r : 0.0);
            }
            const int st = walker_build(items, rates, walkers[which][d]);
            if (st) return st;
        }
    cl.cell_min = water_table(h, lo, error);
    cl.cell_max = water_table(h, hi, error);
    cl.tra = water_table(h, tra, error);
    cl.rel = water_table(h, rel, error);
    cl.bound_upper = water_table(h, upper, error);
    cl.bound_lower = water_table(h, lower, error);
    for (int which = 0; which < 2; ++which)
        for (int d = 0; d < 3; ++d) {
            const HostWalker &hw = walkers[which][d];
            WalkerDev &wd = cl.walker[which][d];
            wd.first_item = water_table(h, hw.first_item, error);
            wd.second_item = water_table(h, hw.second_item, error);
            wd.first_rate = water_table(h, hw.first_rate, error);
            wd.size = (int32_t)hw.first_item.size();
            wd.total_rate = hw.total_rate;
            wd.mean_rate = hw.mean_rate;
        }
    if (error) return error;
    w.cells = cl;
    w.cells_on = 1;
    return JFGPU_OK;
}

extern "C" int jfgpu_water_cells_init(void *water, const JfgpuWaterCellBuffers *buffers, int64_t chains,
                                      void *stream) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h || !buffers || chains < 0 || !h->model.cells_on) return JFGPU_ERROR_ARGUMENT;
    if (chains == 0) return JFGPU_OK;
    if (!buffers->roots || !buffers->occupancy || !buffers->surplus || !buffers->cell_state)
        return JFGPU_ERROR_ARGUMENT;
    const int threads = 128;
    water_cells_init_kernel<<<(unsigned)((chains + threads - 1) / threads), threads, 0,
                              static_cast<cudaStream_t>(stream)>>>(h->model, *buffers, chains);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}

extern "C" int jfgpu_water_cells_run(void *water, double *positions, const double *charges, JfgpuWaterState *state,
                                     const JfgpuWaterCellBuffers *buffers, int64_t chains, int64_t first_chain,
                                     int64_t events, double stop_q, double stop_r, JfgpuEvent *log,
                                     int32_t warps_per_block, void *stream) {
    WaterHandle *h = static_cast<WaterHandle *>(water);
    if (!h || !buffers || chains < 0 || first_chain < 0 || events < 0 || warps_per_block < 0 || warps_per_block > 8 ||
        !h->model.cells_on)
        return JFGPU_ERROR_ARGUMENT;
    if (chains == 0 || events == 0) return JFGPU_OK;
    if (!positions || !charges || !state || !buffers->roots || !buffers->occupancy || !buffers->surplus ||
        !buffers->cell_state)
        return JFGPU_ERROR_ARGUMENT;
    const int warps = warps_per_block ? warps_per_block : 3;
    WaterArgs a;
    memset(&a, 0, sizeof(a));
    a.w = h->model;
    a.positions = positions;
    a.charges = charges;
    a.state = state;
    a.log = log;
    a.chains = chains;
    a.first_chain = first_chain;
    a.events = events;
    a.stop_q = stop_q;
    a.stop_r = stop_r;
    a.roots = buffers->roots;
    a.occ = buffers->occupancy;
    a.sur = buffers->surplus;
    a.cell_state = buffers->cell_state;
    a.root_log = buffers->root_log;
    const size_t shared = water_cells_shared_bytes(h->model.molecules);
    if (shared > 48 * 1024 &&
        cudaFuncSetAttribute(water_cells_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared) !=
            cudaSuccess)
        return JFGPU_ERROR_CUDA;
    water_cells_kernel<<<(unsigned)chains, 32 * warps, shared, static_cast<cudaStream_t>(stream)>>>(a);
    return cudaGetLastError() == cudaSuccess ? JFGPU_OK : JFGPU_ERROR_CUDA;
}
