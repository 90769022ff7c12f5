// host.cpp — host-only parts of the C ABI: parameter defaults, the poly6
// helper, the rest density of a lattice and the seeded block-scene generator.
// None of these touch a GPU, so they work on machines without one.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

#include "../../include/pbf.h"

namespace {

constexpr double kPoly6 = 1.56668147106;  // 315 / (64 pi) as calclambda.glsl:46 writes it

}  // namespace

extern "C" {

int pbf_abi_version(void) { return PBF_ABI_VERSION; }

// SPH::Wpoly6 (src/SPH.cpp:159-164) in double.
double pbf_wpoly6(double r, double h) {
    if (r > h) return 0.0;
    const double t = h * h - r * r;
    double h9 = 1.0;
    for (int i = 0; i < 9; ++i) h9 *= h;
    return kPoly6 * t * t * t / h9;
}

double pbf_rest_density_lattice(double h, double spacing) {
    if (!(h > 0.0) || !(spacing > 0.0)) return 0.0;
    const int m = (int)std::floor(h / spacing) + 1;
    double rho = 0.0;
    for (int a = -m; a <= m; ++a)
        for (int b = -m; b <= m; ++b)
            for (int c = -m; c <= m; ++c) {
                if (a == 0 && b == 0 && c == 0) continue;  // j != i (foreachneighbour.glsl:9)
                const double r = spacing * std::sqrt((double)(a * a + b * b + c * c));
                rho += pbf_wpoly6(r, h);
            }
    return rho;
}

pbf_status pbf_params_default(const uint32_t grid[3], pbf_params* out) {
    if (!grid || !out || grid[0] == 0 || grid[1] == 0 || grid[2] == 0) return PBF_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    // src/SPH.cpp:136-144
    out->one_over_rho_0 = 1.0f;
    out->epsilon = 5.0f;
    out->gravity = 10.0f;
    out->timestep = 0.016f;
    out->tensile_instability_k = 0.1f;
    out->h = 1.0f;  // one cell edge (the reference's h = 2.0 outgrows its 27-cell stencil)
    out->tensile_instability_scale = (float)(1.0 / pbf_wpoly6(0.2, 1.0));
    out->xsph_viscosity_c = 0.01f;
    out->vorticity_epsilon = 5.0f;
    out->num_solver_iterations = 5;  // src/SPH.cpp:25
    out->vorticity_confinement = 0;  // src/SPH.cpp:25
    out->external_force = 0;
    for (int a = 0; a < 3; ++a) out->grid[a] = grid[a];
    // shaders/sph/updatepos.glsl:98-100: wall = (16, 0, 16)
    const float wall[3] = {16.0f, 0.0f, 16.0f};
    for (int a = 0; a < 3; ++a) {
        float lo = wall[a], hi = (float)grid[a] - wall[a];
        if (hi < lo) {  // grid too small for the reference's walls
            lo = 0.0f;
            hi = (float)grid[a];
        }
        out->wall_lo[a] = lo;
        out->wall_hi[a] = hi;
    }
    return PBF_OK;
}

pbf_status pbf_scene_block(const uint32_t lattice[3], float spacing, const float origin[3],
                           float jitter, float vel_uniform, float vel_sigma, uint64_t seed,
                           float* x4, float* v4) {
    if (!lattice || !origin || !x4 || !v4) return PBF_ERR_INVALID_ARGUMENT;
    const uint64_t n = (uint64_t)lattice[0] * lattice[1] * lattice[2];
    std::mt19937_64 rng(seed);
    // uniform double in [0, 1) from the top 53 bits
    auto u01 = [&rng]() { return (double)(rng() >> 11) * (1.0 / 9007199254740992.0); };
    uint64_t id = 0;
    // id order of Simulation::ResetParticleBuffer (src/Simulation.cpp:214-229):
    // x outermost, then z, then y.
    for (uint32_t i = 0; i < lattice[0]; ++i)
        for (uint32_t k = 0; k < lattice[2]; ++k)
            for (uint32_t j = 0; j < lattice[1]; ++j, ++id) {
                const uint32_t idx[3] = {i, j, k};
                for (int a = 0; a < 3; ++a) {
                    const double jit = (2.0 * u01() - 1.0) * (double)jitter;
                    x4[4 * id + a] =
                        (float)((double)origin[a] + (double)spacing * (double)idx[a] + jit);
                }
                x4[4 * id + 3] = 0.0f;
            }
    for (uint64_t p = 0; p < n; ++p) {
        for (int a = 0; a < 3; ++a) {
            double w = 0.0;
            if (vel_uniform > 0.0f) w = (2.0 * u01() - 1.0) * (double)vel_uniform;
            v4[4 * p + a] = (float)w;
        }
        v4[4 * p + 3] = 0.0f;
    }
    if (vel_sigma > 0.0f) {
        // Box-Muller, one normal per uniform pair (cosine branch)
        const double two_pi = 6.283185307179586;
        for (uint64_t p = 0; p < n; ++p)
            for (int a = 0; a < 3; ++a) {
                const double u1 = 1.0 - u01();  // (0, 1]
                const double u2 = u01();
                const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2);
                v4[4 * p + a] = (float)((double)v4[4 * p + a] + (double)vel_sigma * z);
            }
    }
    return PBF_OK;
}

const char* pbf_status_string(pbf_status status) {
    switch (status) {
        case PBF_OK: return "ok";
        case PBF_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PBF_ERR_OUT_OF_MEMORY: return "out of memory";
        case PBF_ERR_CUDA: return "CUDA error";
        case PBF_ERR_DEVICE_FAULT: return "device status error";
        case PBF_ERR_NO_DEVICE: return "no CUDA device";
        case PBF_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

}  // extern "C"
