// jf_engine.cuh -- device-side layout of a chain batch (shared by the engine translation units).
//
// HBM layout (all pools are flat arrays, a chain owns a contiguous slice of each):
//   positions   double[P][3]   FP64 master positions (the reference's Unit.position), chain c at particle_offset
//   positions32 float4[P]      FP32 mirror (x, y, z, charge) read by the FP32 screening
//   charges     double[P]
//   occupancy   int32[O]       cells * max_occupants slots, -1 = empty (SingleActiveCellOccupancy._occupants)
//   cell_slots  float4[O]      cell-ordered FP32 mirror of the occupancy: (x, y, z, identifier bits), bits -1 empty
//   surplus     int32[P]       surplus identifiers of the chain, n_surplus of them (SingleActiveCellOccupancy._surplus)
//   state       JfgpuChainState[C]
// Engine tables (owned by the engine): per-chain ChainDev, per-geometry cell bounds and relative/translate
// tables, per-species far-field bounds (FP64 and FP32), Walker tables and the merged-image Fourier coefficients.
#pragma once
#include <vector>

#include "jf_device.cuh"

namespace jf {

constexpr int kMaxResidues = 64;  // cells per side limit of the near-cell bit mask

struct WalkerDev {
    const int32_t *first_item;
    const int32_t *second_item;
    const double *first_rate;
    int32_t size;
    int32_t pad;
    double total_rate;
    double mean_rate;
};

struct SpeciesDev {
    float lj32[5];               // Lennard-Jones FP32 screening constants: k s^12, -k s^6, 4/k, s^2, r0^2
    MH lj;
    MIC mic;
    const double *bound_upper;   // [cells][3]
    const double *bound_lower;   // [cells][3] negated lower bounds
    const float *bound_upper32;  // [cells][3] FP32 copy for the screening
    float far_rate_max32[3];     // largest FP32 far-field rate by direction (0 without a cell-bounding far field)
    WalkerDev walker[2][3];      // [upper/lower][direction]
    const int4 *mic_terms;       // merged-image sum: real-space images, then Fourier rows (mic_x_warp)
    int mic_images, mic_rows;
    const float *mic_fourier32;  // FP32 copy of the Fourier table (mic_x_warp32)
};

struct ChainDev {
    int32_t potential, far, n, m;
    int32_t ncells, max_occ, n_res, species;
    int32_t initial_active, initial_direction;
    int32_t geom_offset;         // into cell_min / cell_max pools (m entries)
    int32_t table_offset;        // into rel / tra pools (m * m entries)
    int32_t rel_is_mod;          // rel[a][b] == (a - b) mod m and tra[a][b] == (a + b) mod m for every a, b
    int32_t pad0;
    int32_t res[16];             // distinct residues of the neighbour-layer offsets modulo m (n_res of them)
    uint64_t near_mask;          // bit r set when residue r is within the neighbour layers
    int64_t pos_off, occ_off;
    double L, half, side, inv_side, beta, chain_time, speed;
    double diameter_sq;          // hard sphere / hard core: 4 r r (0 = none)
    double bound_prefactor;      // inverse-power Coulomb bound
    double coulomb_prefactor;
    float L32, half32;
    float ulp_margin32;          // rounding scale of FP32 separations (16 L 2^-24): closer calls are flagged
    float screen_abs32;          // absolute screening margin in length units (L 2^-16)
    float speed32, inv_beta32, diameter_sq32, pad32;
    uint64_t key;
};

struct EngineView {
    const ChainDev *chains;
    const SpeciesDev *species;
    const double *cell_min;
    const double *cell_max;
    const int16_t *rel;  // relative_cell index along one axis, [a * m + b]
    const int16_t *tra;  // translate index along one axis, [a * m + b]
};

// host side of a run: CUDA events around the launches when per-kernel timing is on
struct KernelClock {
    virtual ~KernelClock() {}
    virtual void begin(cudaStream_t stream) = 0;            // an event before the next launch on the stream
    virtual void end(cudaStream_t stream, int kind) = 0;    // an event after a launch of this JFGPU_KERNEL_* kind
    int stride = 1;  // the event rounds of the mixed mode that are timed: every stride-th round
};

// streams of a run: the caller's stream, or chain groups on streams of their own forked from it
struct LaunchPlan {
    cudaStream_t stream = nullptr;
    int warps = 4;                          // warps per block of the screening and FP64 kernels
    int groups = 1;                         // chain groups of the mixed mode
    int refine_limit = JFGPU_REFINE_LIST_MAX;  // refine lists longer than this re-solve their event in FP64
    cudaStream_t *group_streams = nullptr;  // [groups] when groups > 1
    cudaEvent_t fork = nullptr;             // recorded on the caller's stream, waited for by every group
    cudaEvent_t *join = nullptr;            // [groups] recorded by every group, waited for by the caller's stream
    KernelClock *clock = nullptr;           // null when timing is off
    void *graphs = nullptr;                 // cache of captured round segments (null: plain launches)
};

// merged-image Coulomb: the Fourier coefficients on the host with the host libm
// (merged_image_coulomb_potential.c:77-119) and the device description pointing at their device copy
std::vector<double> fourier_table(int fc, double alpha, double length);
MIC make_mic(int fc, int pc, double alpha, double length, const double *fourier);
// the real-space images and Fourier rows of the merged-image sum, in the reference's order
void merged_image_terms(int fc, int pc, std::vector<int4> &images, std::vector<int4> &rows);
// exact float bounds of the cells along one axis (cuboid_cells.py:115-131)
void cell_bounds(double length, int m, std::vector<double> &lo, std::vector<double> &hi);
// Walker's alias table on the host in the reference's order (walker.py:53-103)
struct HostWalker {
    std::vector<int32_t> first_item, second_item;
    std::vector<double> first_rate;
    double total_rate = 0.0, mean_rate = 0.0;
};
int walker_build(const std::vector<int> &items, const std::vector<double> &rates, HostWalker &w);
// Lennard-Jones and displaced-even-power parameters as the reference's constructors derive them
MH make_lj(double prefactor, double sigma);
MH make_displaced(double r0, int power, double prefactor);

}  // namespace jf
