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
// reference's acknowledged races (decision Q5: Jacobi order).  The
// vorticity shader's barrier() is honoured by running the dispatch twice: the
// first pass fills the vorticity buffer (phase one of every invocation), the
// second pass reads it complete.
//
// The header SPH builds (src/SPH.cpp:28-60) becomes run-time globals:
// GRID_SIZE, GRID_HASHWEIGHTS = (1, Gx*Gz, Gx), the sphparams fields, h.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <utility>
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

// Switches (off by default) for findcells.glsl:39-43's two boundary cells,
// the oracle's decision Q3: bit 0 gives the first sorted particle's cell its
// start (0), bit 1 the last one's cell its end (n).  The reference never
// writes that end; on a GPU the texture then holds whatever it held, here a
// fresh 0, so the last cell's packed count goes negative and its run reads
// past the particle buffer in some scenes (GL robust access would hide that).
// Bit 1 keeps such a scene's run in bounds; bit 0 separates the first-cell
// quirk from the rest of the reference's behaviour in multi-step comparisons.
int g_cell_fix = 0;

}  // namespace

extern "C" {

int pbfr_record_size(void) { return (int)sizeof(Rec); }

void pbfr_set_cell_fix(int on) { g_cell_fix = on; }

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
    if (g_cell_fix && n > 0) {
        auto texel = [&](const Rec& r) {
            const ivec3 c = ivec3(clamp(vec3(r.x, r.y, r.z), vec3(0.0f, 0.0f, 0.0f), G::GRID_SIZE));
            return (size_t)c.x + (size_t)gx * ((size_t)c.y + (size_t)gy * (size_t)c.z);
        };
        const size_t first = texel(sorted[0]), last = texel(sorted[n - 1]);
        if (g_cell_fix & 1) {
            if (first != 0) start[0] = -1;  // undo thread 0's fixed store
            if (first < cells) start[first] = 0;
        }
        if ((g_cell_fix & 2) && last < cells) end[last] = (int32_t)n;
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

// SurfaceReconstruction's particle passes (src/SurfaceReconstruction.cpp:
// 176-231) with the reference's own vertex and fragment stages: pass 0 runs
// particledepth's vertex and fragment shaders (depth test LESS, cleared to 1,
// gl_FragDepth clamped to [0, 1]); pass 1 runs thickness's vertex shader and,
// for its fragment stage with noise off (thickness/fragment.glsl:122-125),
// discards outside the unit disc and adds 1 (additive blending, cleared to
// 0).  The fixed-function steps between the stages are written out here:
// PointSprite's quad (corners (-1, 1), (1, 1), (1, -1), (-1, -1), triangles
// 0,2,1 and 2,0,3, src/PointSprite.cpp:33-55), the viewport transform, pixel
// centres at i + 1/2 (row 0 at the bottom), the top-left ownership of pixel
// centres on edges, perspective-correct interpolation and near/far clipping.
// V, P: column-major 4x4; out: float[H][W].
int pbfr_splat(int pass, const float* x4, uint32_t n, const float* V, const float* P, uint32_t W,
               uint32_t H, float* out) {
    using namespace glsl;
    mat4 vm, pm;
    for (int c = 0; c < 4; ++c) {
        vm.c[c] = vec4(V[4 * c], V[4 * c + 1], V[4 * c + 2], V[4 * c + 3]);
        pm.c[c] = vec4(P[4 * c], P[4 * c + 1], P[4 * c + 2], P[4 * c + 3]);
    }
    const size_t count = (size_t)W * H;
    for (size_t k = 0; k < count; ++k) out[k] = pass == 0 ? 1.0f : 0.0f;
    struct Corner {
        float x, y, w, cz;
        vec2 t;
        vec3 p;
    };
    const vec2 corner[4] = {vec2(-1.0f, 1.0f), vec2(1.0f, 1.0f), vec2(1.0f, -1.0f), vec2(-1.0f, -1.0f)};
    const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
    auto edge = [](float ax, float ay, float bx, float by, float px, float py) {
        return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
    };
    auto owns = [](float ax, float ay, float bx, float by) { return (ay == by && bx < ax) || by < ay; };
    auto in_edge = [](float e, bool own) { return e > 0.0f || (e == 0.0f && own); };
    for (uint32_t id = 0; id < n; ++id) {
        Corner q[4];
        int near_out = 0, far_out = 0;
        bool skip = false;
        float xmin = 3.0e38f, xmax = -3.0e38f, ymin = 3.0e38f, ymax = -3.0e38f;
        for (int k = 0; k < 4; ++k) {
            vec4 gp;
            vec3 fp;
            vec2 ft;
            if (pass == 0) {
                namespace S = sh_particledepth_vs;
                S::viewmat = vm;
                S::projmat = pm;
                S::vPosition = corner[k];
                S::particlePosition = vec3(x4[4 * id], x4[4 * id + 1], x4[4 * id + 2]);
                S::gl_InstanceID = (int)id;
                S::main_invocation();
                gp = S::gl_Position;
                fp = S::fPosition;
                ft = S::fTexcoord;
            } else {
                namespace S = sh_thickness_vs;
                S::viewmat = vm;
                S::projmat = pm;
                S::vPosition = corner[k];
                S::particlePosition = vec3(x4[4 * id], x4[4 * id + 1], x4[4 * id + 2]);
                S::gl_InstanceID = (int)id;
                S::main_invocation();
                gp = S::gl_Position;
                fp = S::fPosition;
                ft = S::fTexcoord;
            }
            if (!(gp.w > 0.0f)) skip = true;
            near_out += gp.z < -gp.w;
            far_out += gp.z > gp.w;
            q[k] = Corner{hw * (gp.x / gp.w) + hw, hh * (gp.y / gp.w) + hh, gp.w, gp.z, ft, fp};
            xmin = std::fmin(xmin, q[k].x);
            xmax = std::fmax(xmax, q[k].x);
            ymin = std::fmin(ymin, q[k].y);
            ymax = std::fmax(ymax, q[k].y);
        }
        if (skip || near_out == 4 || far_out == 4) continue;
        const bool clip_depth = near_out > 0 || far_out > 0;
        const float fx0 = std::ceil(xmin - 0.5f), fx1 = std::floor(xmax - 0.5f);
        const float fy0 = std::ceil(ymin - 0.5f), fy1 = std::floor(ymax - 0.5f);
        if (!(fx0 <= fx1) || !(fy0 <= fy1)) continue;
        if (fx1 < 0.0f || fy1 < 0.0f || fx0 >= (float)W || fy0 >= (float)H) continue;
        const int x0 = (int)std::fmax(fx0, 0.0f), x1 = (int)std::fmin(fx1, (float)W - 1.0f);
        const int y0 = (int)std::fmax(fy0, 0.0f), y1 = (int)std::fmin(fy1, (float)H - 1.0f);
        const int tri[2][3] = {{0, 2, 1}, {2, 0, 3}};
        for (int ty = y0; ty <= y1; ++ty)
            for (int tx = x0; tx <= x1; ++tx) {
                const float px = (float)tx + 0.5f, py = (float)ty + 0.5f;
                for (int t = 0; t < 2; ++t) {
                    int i0 = tri[t][0], i1 = tri[t][1], i2 = tri[t][2];
                    float area = edge(q[i0].x, q[i0].y, q[i1].x, q[i1].y, q[i2].x, q[i2].y);
                    if (area == 0.0f || area != area) continue;
                    if (area < 0.0f) {
                        std::swap(i1, i2);
                        area = -area;
                    }
                    const Corner &a = q[i0], &b = q[i1], &c = q[i2];
                    const float e0 = edge(b.x, b.y, c.x, c.y, px, py);
                    const float e1 = edge(c.x, c.y, a.x, a.y, px, py);
                    const float e2 = edge(a.x, a.y, b.x, b.y, px, py);
                    if (!in_edge(e0, owns(b.x, b.y, c.x, c.y)) || !in_edge(e1, owns(c.x, c.y, a.x, a.y)) ||
                        !in_edge(e2, owns(a.x, a.y, b.x, b.y)))
                        continue;
                    const float l0 = (e0 / area) / a.w, l1 = (e1 / area) / b.w, l2 = (e2 / area) / c.w;
                    const float ls = (l0 + l1) + l2;
                    auto lerp = [&](float A, float B, float C) { return ((l0 * A + l1 * B) + l2 * C) / ls; };
                    if (clip_depth) {
                        const float zc = lerp(a.cz, b.cz, c.cz), wc = lerp(a.w, b.w, c.w);
                        if (zc < -wc || zc > wc) break;
                    }
                    const vec2 tc(lerp(a.t.x, b.t.x, c.t.x), lerp(a.t.y, b.t.y, c.t.y));
                    const size_t pix = (size_t)ty * W + tx;
                    if (pass == 0) {
                        namespace S = sh_particledepth_fs;
                        S::viewmat = vm;
                        S::projmat = pm;
                        S::fTexcoord = tc;
                        S::fPosition = vec3(lerp(a.p.x, b.p.x, c.p.x), lerp(a.p.y, b.p.y, c.p.y),
                                            lerp(a.p.z, b.p.z, c.p.z));
                        S::discarded = false;
                        S::main_invocation();
                        if (S::discarded) break;
                        float d = S::gl_FragDepth;
                        if (d != d) break;
                        d = d < 0.0f ? 0.0f : (d > 1.0f ? 1.0f : d);
                        if (d < out[pix]) out[pix] = d;
                    } else {
                        if (dot(tc, tc) > 1) break;  // thickness/fragment.glsl:122-125
                        out[pix] += 1.0f;
                    }
                    break;
                }
            }
    }
    return 0;
}

int pbfr_substep(const Params* p, uint32_t n, float* x4, float* v4, uint32_t* out_ids,
                 int32_t* out_start, int32_t* out_end, int32_t* out_nbr, float* out_lambda) {
    return pbfr_substep_highlight(p, n, x4, v4, out_ids, out_start, out_end, out_nbr, out_lambda,
                                  nullptr);
}

}  // extern "C"
