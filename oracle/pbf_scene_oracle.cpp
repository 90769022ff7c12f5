// pbf_scene_oracle.cpp — the workloads' seeded scenes and constants on the
// oracle side (TEST INFRASTRUCTURE ONLY).
//
// The CPU reference arm of bench.py and the tests build their scenes through
// these functions, so that timing the reference path never loads the product
// library.  They follow the same published recipe as the product's scene
// generator, and tests/test_oracle.py checks the two byte for byte:
//   - lattice block in Simulation::ResetParticleBuffer's id order
//     (src/Simulation.cpp:214-229: x outermost, then z, then y);
//   - std::mt19937_64 seeded with the 64-bit seed; a uniform double in [0, 1)
//     from the top 53 bits of each draw;
//   - position = origin + spacing * index + jitter * (2u - 1), per axis, all
//     positions first, then the uniform velocities (2u - 1) * vel_uniform,
//     then, if vel_sigma > 0, one Box-Muller normal (cosine branch, from
//     u1 = 1 - u, u2 = u) added per velocity component;
//   - Wpoly6 (src/SPH.cpp:159-164) in double, and the rest density of an
//     unjittered interior lattice point with the self term left out
//     (foreachneighbour.glsl:9);
//   - SPH's defaults (src/SPH.cpp:25-26,136-144; walls updatepos.glsl:98-100).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

#include "pbf_oracle.hpp"

namespace {

double poly6_double(double r, double h) {
    if (r > h) return 0.0;
    const double q = h * h - r * r;
    return 1.56668147106 * q * q * q / (h * h * h * h * h * h * h * h * h);
}

struct Uniform01 {
    std::mt19937_64 g;
    explicit Uniform01(uint64_t seed) : g(seed) {}
    double operator()() { return (double)(g() >> 11) * 0x1.0p-53; }
};

}  // namespace

extern "C" {

double pbfo_wpoly6(double r, double h) { return poly6_double(r, h); }

double pbfo_rest_density_lattice(double h, double spacing) {
    if (!(h > 0.0) || !(spacing > 0.0)) return 0.0;
    const int reach = (int)std::floor(h / spacing) + 1;
    double sum = 0.0;
    for (int a = -reach; a <= reach; ++a)
        for (int b = -reach; b <= reach; ++b)
            for (int c = -reach; c <= reach; ++c) {
                const int q = a * a + b * b + c * c;
                if (q == 0) continue;
                sum += poly6_double(spacing * std::sqrt((double)q), h);
            }
    return sum;
}

int pbfo_params_default(const uint32_t grid[3], pbfo::Params* p) {
    if (!grid || !p || !grid[0] || !grid[1] || !grid[2]) return 1;
    std::memset(p, 0, sizeof(*p));
    p->one_over_rho_0 = 1.0f;
    p->epsilon = 5.0f;
    p->gravity = 10.0f;
    p->timestep = 0.016f;
    p->tensile_instability_k = 0.1f;
    p->h = 1.0f;
    p->tensile_instability_scale = (float)(1.0 / poly6_double(0.2, 1.0));
    p->xsph_viscosity_c = 0.01f;
    p->vorticity_epsilon = 5.0f;
    p->num_solver_iterations = 5;
    p->vorticity_confinement = 0;
    p->external_force = 0;
    const float wall[3] = {16.0f, 0.0f, 16.0f};
    for (int a = 0; a < 3; ++a) {
        p->grid[a] = grid[a];
        const bool fits = (float)grid[a] - wall[a] >= wall[a];
        p->wall_lo[a] = fits ? wall[a] : 0.0f;
        p->wall_hi[a] = fits ? (float)grid[a] - wall[a] : (float)grid[a];
    }
    return 0;
}

int pbfo_scene_block(const uint32_t lattice[3], float spacing, const float origin[3], float jitter,
                     float vel_uniform, float vel_sigma, uint64_t seed, float* x4, float* v4) {
    if (!lattice || !origin || !x4 || !v4) return 1;
    const uint64_t n = (uint64_t)lattice[0] * lattice[1] * lattice[2];
    Uniform01 u(seed);
    float* px = x4;
    for (uint32_t i = 0; i < lattice[0]; ++i)
        for (uint32_t k = 0; k < lattice[2]; ++k)
            for (uint32_t j = 0; j < lattice[1]; ++j, px += 4) {
                const uint32_t ijk[3] = {i, j, k};
                for (int a = 0; a < 3; ++a) {
                    const double d = (double)jitter * (2.0 * u() - 1.0);
                    px[a] = (float)((double)origin[a] + (double)spacing * (double)ijk[a] + d);
                }
                px[3] = 0.0f;
            }
    for (uint64_t q = 0; q < 4 * n; q += 4) {
        for (int a = 0; a < 3; ++a)
            v4[q + a] = vel_uniform > 0.0f ? (float)((double)vel_uniform * (2.0 * u() - 1.0)) : 0.0f;
        v4[q + 3] = 0.0f;
    }
    if (vel_sigma > 0.0f)
        for (uint64_t q = 0; q < 4 * n; q += 4)
            for (int a = 0; a < 3; ++a) {
                const double u1 = 1.0 - u();
                const double u2 = u();
                const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
                v4[q + a] = (float)((double)v4[q + a] + (double)vel_sigma * z);
            }
    return 0;
}

}  // extern "C"
