// splat.cu — headless particle splatting: SurfaceReconstruction's two
// particle passes (src/SurfaceReconstruction.cpp:176-231) as CUDA kernels
// writing device buffers instead of GL framebuffers.
//
//  depth      shaders/particledepth/{vertex,fragment}.glsl: each particle is a
//             view-aligned quad of half-size 0.1 (two triangles, PointSprite's
//             indices 0,2,1 / 2,0,3, src/PointSprite.cpp:33-55); a fragment
//             inside the unit disc of its texture coordinate writes the
//             depth of the sphere surface, clip z / clip w, clamped to
//             [0, 1]; the depth test keeps the smallest (cleared to 1).
//  thickness  shaders/thickness/{vertex,fragment}.glsl with noise off: every
//             fragment inside the disc adds 1 (additive blending, no depth
//             test; cleared to 0).
//
// Rasterisation follows the GL rules the reference relies on: the viewport
// transform xw = (W/2) xd + W/2, pixel centres at (i + 1/2, j + 1/2), row 0
// at the bottom, a pixel centre on a shared edge owned by exactly one
// triangle (top-left rule in window coordinates with y up), attributes
// interpolated perspective-correctly, and primitives clipped to the near and
// far planes (-w <= z <= w).  Every floating-point step is one explicitly
// rounded operation in a fixed order, so the CPU oracle reproduces the
// output bit for bit; both outputs are order-independent (a minimum and an
// exact count), so thread scheduling cannot change them.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pbf.h"
#include "internal.h"
#include "sim.h"

namespace pbf {
namespace {

__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

struct View {
    float V[16], P[16];  // column-major: m[4 * column + row]
};

// mat4 * vec4 as GLSL evaluates it: column 0 * x + column 1 * y + column 2 * z
// + column 3 * w, summed left to right, one rounding per operation.
__device__ __forceinline__ float4 mul4(const float* m, float4 v) {
    float4 r;
    r.x = fa(fa(fa(fm(m[0], v.x), fm(m[4], v.y)), fm(m[8], v.z)), fm(m[12], v.w));
    r.y = fa(fa(fa(fm(m[1], v.x), fm(m[5], v.y)), fm(m[9], v.z)), fm(m[13], v.w));
    r.z = fa(fa(fa(fm(m[2], v.x), fm(m[6], v.y)), fm(m[10], v.z)), fm(m[14], v.w));
    r.w = fa(fa(fa(fm(m[3], v.x), fm(m[7], v.y)), fm(m[11], v.z)), fm(m[15], v.w));
    return r;
}

struct Vert {
    float x, y;        // window coordinates
    float w;           // clip w (perspective-correct interpolation)
    float cz;          // clip z (near / far clipping of straddling primitives)
    float tx, ty;      // fTexcoord
    float px, py, pz;  // fPosition (view space)
};

// Edge function of (a -> b) at p, in window coordinates.
__device__ __forceinline__ float edge(float ax, float ay, float bx, float by, float px, float py) {
    return fs(fm(fs(bx, ax), fs(py, ay)), fm(fs(by, ay), fs(px, ax)));
}

// Does a pixel centre exactly on edge (a -> b) of a counter-clockwise
// triangle (y up) belong to it?  Top edges (horizontal, traversed towards -x)
// and left edges (traversed towards -y) do.
__device__ __forceinline__ bool owns_edge(float ax, float ay, float bx, float by) {
    return (ay == by && bx < ax) || by < ay;
}

__device__ __forceinline__ bool inside(float e, bool own) { return e > 0.0f || (e == 0.0f && own); }

template <int PASS>
__global__ void __launch_bounds__(128)
k_splat(const float4* __restrict__ pos, uint32_t n, View view, uint32_t W, uint32_t H,
        float* __restrict__ out) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const float4 p4 = pos[id];
    // vertex shader: world position 0.2 p + 0.2 (-64, 1, -64) (vertex.glsl:41/42)
    const float4 c = make_float4(fa(fm(0.2f, p4.x), fm(0.2f, -64.0f)), fa(fm(0.2f, p4.y), fm(0.2f, 1.0f)),
                                 fa(fm(0.2f, p4.z), fm(0.2f, -64.0f)), 1.0f);
    const float4 m = mul4(view.V, c);
    // the corner offset's w: depth adds vec4(0.1 v, 0, 1), thickness adds
    // vec4(v, 0, 1) * 0.1 (the reference's w quirks, kept)
    const float ow = PASS == PBF_SPLAT_DEPTH ? 1.0f : 0.1f;
    const float hw = fm(0.5f, (float)W), hh = fm(0.5f, (float)H);
    Vert q[4];
    const float cvx[4] = {-1.0f, 1.0f, 1.0f, -1.0f}, cvy[4] = {1.0f, 1.0f, -1.0f, -1.0f};
    int near_out = 0, far_out = 0;
    float xmin = 3.0e38f, xmax = -3.0e38f, ymin = 3.0e38f, ymax = -3.0e38f;
    for (int k = 0; k < 4; ++k) {
        const float4 ps = make_float4(fa(m.x, fm(0.1f, cvx[k])), fa(m.y, fm(0.1f, cvy[k])), fa(m.z, 0.0f),
                                      fa(m.w, ow));
        const float4 cl = mul4(view.P, ps);
        if (!(cl.w > 0.0f)) return;  // a corner at or behind the eye: not drawn
        near_out += cl.z < -cl.w;
        far_out += cl.z > cl.w;
        Vert& v = q[k];
        v.x = fa(fm(hw, fd(cl.x, cl.w)), hw);
        v.y = fa(fm(hh, fd(cl.y, cl.w)), hh);
        v.w = cl.w;
        v.cz = cl.z;
        v.tx = cvx[k];
        v.ty = cvy[k];
        v.px = ps.x;
        v.py = ps.y;
        v.pz = ps.z;
        xmin = fminf(xmin, v.x);
        xmax = fmaxf(xmax, v.x);
        ymin = fminf(ymin, v.y);
        ymax = fmaxf(ymax, v.y);
    }
    if (near_out == 4 || far_out == 4) return;
    const bool clip_depth = near_out > 0 || far_out > 0;
    // pixel centres i + 0.5 inside [xmin, xmax]
    const float fx0 = ceilf(xmin - 0.5f), fx1 = floorf(xmax - 0.5f);
    const float fy0 = ceilf(ymin - 0.5f), fy1 = floorf(ymax - 0.5f);
    if (!(fx0 <= fx1) || !(fy0 <= fy1)) return;
    if (fx1 < 0.0f || fy1 < 0.0f || fx0 >= (float)W || fy0 >= (float)H) return;
    const int x0 = (int)fmaxf(fx0, 0.0f), x1 = (int)fminf(fx1, (float)W - 1.0f);
    const int y0 = (int)fmaxf(fy0, 0.0f), y1 = (int)fminf(fy1, (float)H - 1.0f);
    // the two triangles (PointSprite indices 0,2,1 and 2,0,3), made
    // counter-clockwise in window coordinates
    const int tri[2][3] = {{0, 2, 1}, {2, 0, 3}};
    for (int ty = y0; ty <= y1; ++ty) {
        const float py = (float)ty + 0.5f;
        for (int tx = x0; tx <= x1; ++tx) {
            const float px = (float)tx + 0.5f;
            for (int t = 0; t < 2; ++t) {
                int i0 = tri[t][0], i1 = tri[t][1], i2 = tri[t][2];
                float area = edge(q[i0].x, q[i0].y, q[i1].x, q[i1].y, q[i2].x, q[i2].y);
                if (area == 0.0f || area != area) continue;
                if (area < 0.0f) {
                    const int s = i1;
                    i1 = i2;
                    i2 = s;
                    area = -area;
                }
                const Vert &a = q[i0], &b = q[i1], &cc = q[i2];
                const float e0 = edge(b.x, b.y, cc.x, cc.y, px, py);  // opposite a
                const float e1 = edge(cc.x, cc.y, a.x, a.y, px, py);  // opposite b
                const float e2 = edge(a.x, a.y, b.x, b.y, px, py);    // opposite c
                if (!inside(e0, owns_edge(b.x, b.y, cc.x, cc.y)) ||
                    !inside(e1, owns_edge(cc.x, cc.y, a.x, a.y)) ||
                    !inside(e2, owns_edge(a.x, a.y, b.x, b.y)))
                    continue;
                // perspective-correct barycentric weights
                const float l0 = fd(fd(e0, area), a.w), l1 = fd(fd(e1, area), b.w),
                            l2 = fd(fd(e2, area), cc.w);
                const float ls = fa(fa(l0, l1), l2);
                auto interp = [&](float A, float B, float C) {
                    return fd(fa(fa(fm(l0, A), fm(l1, B)), fm(l2, C)), ls);
                };
                if (clip_depth) {
                    const float zc = interp(a.cz, b.cz, cc.cz), wc = interp(a.w, b.w, cc.w);
                    if (zc < -wc || zc > wc) break;
                }
                const float u = interp(a.tx, b.tx, cc.tx), v = interp(a.ty, b.ty, cc.ty);
                // fragment shader: r = dot(t, t); discard outside the disc
                const float r = fa(fm(u, u), fm(v, v));
                if (r > 1.0f) break;
                if (PASS == PBF_SPLAT_THICKNESS) {
                    atomicAdd(out + (size_t)ty * W + tx, 1.0f);
                } else {
                    // normal = (t, -sqrt(1 - r)); fPos = fPosition - 0.1 normal;
                    // depth = (P fPos).z / (P fPos).w  (particledepth/fragment.glsl:40-46)
                    const float nz = -__fsqrt_rn(fs(1.0f, r));
                    const float4 fp = make_float4(fs(interp(a.px, b.px, cc.px), fm(0.1f, u)),
                                                  fs(interp(a.py, b.py, cc.py), fm(0.1f, v)),
                                                  fs(interp(a.pz, b.pz, cc.pz), fm(0.1f, nz)), 1.0f);
                    const float4 cp = mul4(view.P, fp);
                    float d = fd(cp.z, cp.w);
                    if (d != d) break;  // NaN fragments are dropped
                    d = d < 0.0f ? 0.0f : (d > 1.0f ? 1.0f : d);
                    atomicMin(reinterpret_cast<unsigned int*>(out) + (size_t)ty * W + tx,
                              __float_as_uint(d));
                }
                break;  // a pixel centre belongs to at most one of the two triangles
            }
        }
    }
}

__global__ void k_fill(float* __restrict__ out, size_t count, float value) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = value;
}

}  // namespace
}  // namespace pbf

extern "C" pbf_status pbf_splat(int pass, const float* positions, uint32_t n, const pbf_view* view,
                                uint32_t width, uint32_t height, float* out, void* stream) {
    pbf::NvtxRange nvtx_("pbf_splat");
    using namespace pbf;
    if (pass != PBF_SPLAT_DEPTH && pass != PBF_SPLAT_THICKNESS)
        return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "pass must be PBF_SPLAT_DEPTH or PBF_SPLAT_THICKNESS");
    if (!view || !out || (n > 0 && !positions))
        return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(nullptr, PBF_ERR_INVALID_ARGUMENT, "width and height must be in [1, 16384]");
    cudaStream_t st = (cudaStream_t)stream;
    View v;
    for (int k = 0; k < 16; ++k) {
        v.V[k] = view->viewmat[k];
        v.P[k] = view->projmat[k];
    }
    const size_t count = (size_t)width * height;
    k_fill<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(out, count,
                                                            pass == PBF_SPLAT_DEPTH ? 1.0f : 0.0f);
    if (n > 0) {
        const unsigned g = (n + 127) / 128;
        if (pass == PBF_SPLAT_DEPTH)
            k_splat<PBF_SPLAT_DEPTH><<<g, 128, 0, st>>>((const float4*)positions, n, v, width, height, out);
        else
            k_splat<PBF_SPLAT_THICKNESS><<<g, 128, 0, st>>>((const float4*)positions, n, v, width, height,
                                                            out);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "pbf_splat");
    return PBF_OK;
}
