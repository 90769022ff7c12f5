// ref_driver.cpp — runs the reference's own compute shaders (compiled as C++
// by oracle/ref_build.py) in the dispatch order of SPH::Run
// (src/SPH.cpp:246-334), one invocation after another.  TEST INFRASTRUCTURE
// ONLY: it pins the oracle to the reference's code.
//
// Dispatch semantics.  Invocations run sequentially.  Where a shader writes
// an element other invocations of the same dispatch read (updatepos writes
// particlekeys in place, updatepos.glsl:53-55,104; vorticity writes the
// velocity image and the vorticity buffer it also reads, vorticity.glsl:50,
// 60-72, 85), each invocation's own write is held back until the dispatch
// ends, so every read sees the dispatch's input: the Jacobi reading of the
// reference's acknowledged races (decision Q5 of oracle/README.md).  The
// vorticity shader's barrier() is honoured by running the dispatch twice: the
// first pass fills the vorticity buffer (phase one of every invocation), the
// second pass reads it complete.
//
// The header SPH builds (src/SPH.cpp:28-60) becomes run-time globals:
// GRID_SIZE, GRID_HASHWEIGHTS = (1, Gx*Gz, Gx), the sphparams fields, h.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "glsl.hpp"

namespace refglobals {
using glsl::ivec3;
using glsl::uvec3;
using glsl::vec3;
vec3 GRID_SIZE;
ivec3 GRID_HASHWEIGHTS;
float one_over_rho_0, epsilon, gravity, timestep, tensile_instability_k, tensile_instability_scale,
    xsph_viscosity_c, vorticity_epsilon;
float h;
uvec3 gl_GlobalInvocationID;
}  // namespace refglobals

#include "gen_shaders.inc"

namespace {

// Same layout as pbf_params (include/pbf.h).
struct Params {
    float one_over_rho_0, epsilon, gravity, timestep, tensile_instability_k,
        tensile_instability_scale, xsph_viscosity_c, vorticity_epsilon, h;
    uint32_t num_solver_iterations, vorticity_confinement, external_force;
    uint32_t grid[3];
    float wall_lo[3], wall_hi[3];
};

void set_invocation(uint32_t gid) { refglobals::gl_GlobalInvocationID = {gid, 0u, 0u}; }

uint32_t count_sortbits(uint64_t v) {  // src/RadixSort.cpp:24-30
    uint32_t r = 1;
    while (v >>= 1) r++;
    return r;
}

struct Rec {
    float x, y, z;
    int32_t id;
};
static_assert(sizeof(Rec) == 16, "particle key record");

}  // namespace

extern "C" {

int pbfr_record_size(void) { return (int)sizeof(Rec); }

// One substep.  x4, v4 (float4, id order) are updated in place.  Optional
// outputs: sorted ids [n], grid start/end textures [Gx*Gy*Gz] (x fastest,
// then y, then z: the 3-D texture layout), the packed neighbour texture
// [12 n] (start | count << 24, 3 ivec4 per sorted particle), lambda of the
// last iteration [n] (sorted).  highlight (uint32[n], id order, may be NULL)
// goes through the clearhighlight and highlight dispatches, which SPH::Run
// issues after the neighbour search (src/SPH.cpp:288-297).
int pbfr_substep_highlight(const Params* p, uint32_t n, float* x4, float* v4, uint32_t* out_ids,
                           int32_t* out_start, int32_t* out_end, int32_t* out_nbr,
                           float* out_lambda, uint32_t* highlight) {
    using namespace glsl;
    namespace G = refglobals;
    const int gx = (int)p->grid[0], gy = (int)p->grid[1], gz = (int)p->grid[2];
    G::GRID_SIZE = vec3((float)gx, (float)gy, (float)gz);
    G::GRID_HASHWEIGHTS = ivec3(1, gx * gz, gx);
    G::one_over_rho_0 = p->one_over_rho_0;
    G::epsilon = p->epsilon;
    G::gravity = p->gravity;
    G::timestep = p->timestep;
    G::tensile_instability_k = p->tensile_instability_k;
    G::tensile_instability_scale = p->tensile_instability_scale;
    G::xsph_viscosity_c = p->xsph_viscosity_c;
    G::vorticity_epsilon = p->vorticity_epsilon;
    G::h = p->h;
    const size_t cells = (size_t)gx * gy * gz;

    // 1 predictpos
    std::vector<Rec> keys(n);
    sh_predictpos::particlekeys = reinterpret_cast<sh_predictpos::ParticleKey*>(keys.data());
    sh_predictpos::positiontexture = samplerBuffer{x4, 4};
    sh_predictpos::velocitytexture = samplerBuffer{v4, 4};
    sh_predictpos::extforce = p->external_force != 0;
    for (uint32_t g = 0; g < n; ++g) {
        set_invocation(g);
        sh_predictpos::main_invocation();
    }

    // 2 sort by GetHash over the bits RadixSort sorts (src/RadixSort.cpp:44,124-133)
    const uint32_t numbits = count_sortbits((uint64_t)cells - 1);
    const uint32_t sorted_bits = 2 * ((numbits + 1) >> 1);
    const uint32_t mask = sorted_bits >= 32 ? 0xFFFFFFFFu : ((1u << sorted_bits) - 1u);
    std::vector<uint32_t> hash(n), order(n);
    for (uint32_t i = 0; i < n; ++i)
        hash[i] = sh_hash::GetHash(vec3(keys[i].x, keys[i].y, keys[i].z)) & mask;
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return hash[a] < hash[b]; });
    std::vector<Rec> sorted(n);
    for (uint32_t i = 0; i < n; ++i) sorted[i] = keys[order[i]];

    // 3 findcells (start cleared to -1 each substep, end never cleared:
    //   src/NeighbourCellFinder.cpp:113-126) and neighbourcells
    std::vector<int32_t> start(cells, -1), end(cells, 0), nbr(12ull * n, 0);
    sh_findcells::particlekeys = reinterpret_cast<vec4*>(sorted.data());
    sh_findcells::gridtexture = iimage3D{start.data(), gx, gy, gz};
    sh_findcells::gridendtexture = iimage3D{end.data(), gx, gy, gz};
    for (uint32_t g = 0; g < n; ++g) {
        set_invocation(g);
        sh_findcells::main_invocation();
    }
    sh_neighbourcells::particlekeys = reinterpret_cast<vec4*>(sorted.data());
    sh_neighbourcells::gridtexture = isampler3D{start.data(), gx, gy, gz};
    sh_neighbourcells::gridendtexture = isampler3D{end.data(), gx, gy, gz};
    sh_neighbourcells::neighbourtexture = iimageBuffer{nbr.data()};
    for (uint32_t g = 0; g < n; ++g) {
        set_invocation(g);
        sh_neighbourcells::main_invocation();
    }

    // particle highlighting (each invocation's atomics land at once; the
    // highlight shader only reads bit 0, which no invocation changes)
    if (highlight) {
        sh_clearhighlight::highlighttexture = uimageBuffer{highlight};
        for (uint32_t g = 0; g < n; ++g) {
            set_invocation(g);
            sh_clearhighlight::main_invocation();
        }
        sh_highlight::particlekeys = reinterpret_cast<sh_highlight::ParticleKey*>(sorted.data());
        sh_highlight::neighbourcelltexture = isamplerBuffer{nbr.data()};
        sh_highlight::highlighttexture = uimageBuffer{highlight};
        for (uint32_t g = 0; g < n; ++g) {
            set_invocation(g);
            sh_highlight::main_invocation();
        }
    }

    // 4 solver iterations
    std::vector<float> lambda(n, 0.0f);
    std::vector<Rec> next(n);
    for (uint32_t it = 0; it < p->num_solver_iterations; ++it) {
        sh_calclambda::particlekeys = reinterpret_cast<sh_calclambda::ParticleKey*>(sorted.data());
        sh_calclambda::neighbourcelltexture = isamplerBuffer{nbr.data()};
        sh_calclambda::lambdatexture = imageBuffer{lambda.data(), 1};
        for (uint32_t g = 0; g < n; ++g) {
            set_invocation(g);
            sh_calclambda::main_invocation();
        }
        sh_updatepos::particlekeys = reinterpret_cast<sh_updatepos::ParticleKey*>(sorted.data());
        sh_updatepos::neighbourcelltexture = isamplerBuffer{nbr.data()};
        sh_updatepos::lambdatexture = samplerBuffer{lambda.data(), 1};
        for (uint32_t g = 0; g < n; ++g) {
            const Rec keep = sorted[g];
            set_invocation(g);
            sh_updatepos::main_invocation();
            next[g] = sorted[g];
            sorted[g] = keep;  // the write lands when the dispatch ends
        }
        sorted.swap(next);
    }

    // 5 update (each invocation reads and writes only its own id)
    sh_update::particlekeys = reinterpret_cast<sh_update::ParticleKey*>(sorted.data());
    sh_update::positiontexture = imageBuffer{x4, 4};
    sh_update::velocitytexture = imageBuffer{v4, 4};
    for (uint32_t g = 0; g < n; ++g) {
        set_invocation(g);
        sh_update::main_invocation();
    }

    // vorticity (+ XSPH), when enabled (src/SPH.cpp:325-331)
    if (p->vorticity_confinement) {
        std::vector<float> vort_a(n, 0.0f), vout(4ull * n);
        sh_vorticity::particlekeys = reinterpret_cast<vec4*>(sorted.data());
        sh_vorticity::neighbourcelltexture = isamplerBuffer{nbr.data()};
        sh_vorticity::velocitytexture = imageBuffer{v4, 4};
        for (int pass = 0; pass < 2; ++pass) {
            std::vector<float> vort_b = vort_a;
            sh_vorticity::vorticities = pass == 0 ? vort_a.data() : vort_b.data();
            for (uint32_t g = 0; g < n; ++g) {
                const int32_t pid = sorted[g].id;
                float keep[4];
                std::copy(v4 + 4ull * pid, v4 + 4ull * pid + 4, keep);
                set_invocation(g);
                sh_vorticity::main_invocation();
                std::copy(v4 + 4ull * pid, v4 + 4ull * pid + 4, vout.begin() + 4ull * pid);
                std::copy(keep, keep + 4, v4 + 4ull * pid);
            }
        }
        std::copy(vout.begin(), vout.end(), v4);
    }

    if (out_ids)
        for (uint32_t i = 0; i < n; ++i) out_ids[i] = (uint32_t)sorted[i].id;
    if (out_start) std::copy(start.begin(), start.end(), out_start);
    if (out_end) std::copy(end.begin(), end.end(), out_end);
    if (out_nbr) std::copy(nbr.begin(), nbr.end(), out_nbr);
    if (out_lambda) std::copy(lambda.begin(), lambda.end(), out_lambda);
    return 0;
}

int pbfr_substep(const Params* p, uint32_t n, float* x4, float* v4, uint32_t* out_ids,
                 int32_t* out_start, int32_t* out_end, int32_t* out_nbr, float* out_lambda) {
    return pbfr_substep_highlight(p, n, x4, v4, out_ids, out_start, out_end, out_nbr, out_lambda,
                                  nullptr);
}

}  // extern "C"
