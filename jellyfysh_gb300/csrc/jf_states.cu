// jf_states.cu -- seeded initial states of the batched workloads, on the host.
//
// The reference places its atoms uniformly at random without overlap rejection
// (jellyfysh/input_output_handler/input_handler/random_node_creator/atom_random_node_creator.py:56-67), so the hard
// sphere starts of the batched workloads are generated here: random sequential addition (uniform trial points in the
// periodic cube, a trial closer than one diameter to a placed sphere, minimum image, is rejected).  Trials are tested
// against the spheres of the neighbouring cells of a grid whose cells are at least one diameter wide, so that the
// thousands of chains of up to a few thousand spheres near the RSA jamming density start in seconds.
#include <cmath>
#include <cstdint>
#include <vector>

#include "jfgpu.h"

namespace {

// SplitMix64 (Steele, Lea and Flood 2014): the trial points' generator
struct SplitMix {
    uint64_t state;
    uint64_t next() {
        uint64_t z = (state += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
};

}  // namespace

extern "C" int jfgpu_random_sequential_addition(int64_t n, double radius, double system_length, uint64_t seed,
                                                int64_t max_trials, double *positions) {
    if (n < 0 || !(radius >= 0.0) || !(system_length > 0.0) || !positions || max_trials < 0) return JFGPU_ERROR_ARGUMENT;
    const double diameter = 2.0 * radius;
    const double diameter_sq = diameter * diameter;
    const double half = system_length / 2.0;
    long long g = diameter > 0.0 ? (long long)std::floor(system_length / diameter) : 1;
    if (g < 1) g = 1;
    if (g > 256) g = 256;
    const double inv_side = (double)g / system_length;
    std::vector<int64_t> head((size_t)(g * g * g), -1), next((size_t)n, -1);
    SplitMix rng{seed};
    int64_t placed = 0, trials = 0;
    auto cell_axis = [&](double x) {
        long long i = (long long)(x * inv_side);
        return i >= g ? g - 1 : (i < 0 ? 0 : i);
    };
    // neighbouring cells along one axis: three when the grid has at least three cells, else all of them
    const long long span = g >= 3 ? 1 : 0;
    while (placed < n) {
        if (trials++ >= max_trials) return JFGPU_ERROR_TABLE;
        double p[3];
        for (int k = 0; k < 3; ++k) {
            p[k] = system_length * rng.uniform();
            if (p[k] >= system_length) p[k] = 0.0;
        }
        const long long c[3] = {cell_axis(p[0]), cell_axis(p[1]), cell_axis(p[2])};
        bool overlap = false;
        for (long long dz = (g >= 3 ? -span : 0); dz <= (g >= 3 ? span : g - 1) && !overlap; ++dz)
            for (long long dy = (g >= 3 ? -span : 0); dy <= (g >= 3 ? span : g - 1) && !overlap; ++dy)
                for (long long dx = (g >= 3 ? -span : 0); dx <= (g >= 3 ? span : g - 1) && !overlap; ++dx) {
                    const long long x = g >= 3 ? (c[0] + dx + g) % g : dx;
                    const long long y = g >= 3 ? (c[1] + dy + g) % g : dy;
                    const long long z = g >= 3 ? (c[2] + dz + g) % g : dz;
                    for (int64_t j = head[(size_t)(x + g * (y + g * z))]; j >= 0 && !overlap; j = next[(size_t)j]) {
                        double d2 = 0.0;
                        for (int k = 0; k < 3; ++k) {
                            double s = positions[3 * j + k] - p[k];
                            if (s > half) s -= system_length;
                            if (s < -half) s += system_length;
                            d2 += s * s;
                        }
                        if (d2 < diameter_sq) overlap = true;
                    }
                }
        if (overlap) continue;
        for (int k = 0; k < 3; ++k) positions[3 * placed + k] = p[k];
        const size_t cell = (size_t)(c[0] + g * (c[1] + g * c[2]));
        next[(size_t)placed] = head[cell];
        head[cell] = placed;
        ++placed;
    }
    return JFGPU_OK;
}
