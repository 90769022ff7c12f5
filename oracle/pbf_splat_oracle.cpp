// pbf_splat_oracle.cpp — CPU restatement of SurfaceReconstruction's two
// particle passes (TEST INFRASTRUCTURE: the checker of pbf_splat).
//
//   depth      shaders/particledepth/vertex.glsl:41-46, fragment.glsl:36-46
//   thickness  shaders/thickness/vertex.glsl:42-48, fragment.glsl:122-125
//              (noise off, SurfaceReconstruction.cpp:189-208)
//   draw       PointSprite's quad, indices 0,2,1 / 2,0,3 (src/PointSprite.cpp:33-55)
//
// The GL pipeline steps the shaders rely on are restated with the rules
// written out: mat4 * vec4 as a left-to-right sum of column terms; viewport
// xw = (W/2) xd + W/2; pixel centres at i + 1/2 with row 0 at the bottom; a
// pixel centre on an edge belongs to the counter-clockwise triangle for which
// the edge is a top or left edge (y up); perspective-correct attribute
// interpolation; near/far clipping (-w <= z <= w); the depth test LESS against
// a buffer cleared to 1 with fragment depths clamped to [0, 1]; additive
// blending into a buffer cleared to 0.  Compiled with -ffp-contract=off: one
// IEEE rounding per operation, in the order written.
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

struct V4 {
    float x, y, z, w;
};

V4 mul4(const float* m, V4 v) {
    V4 r;
    r.x = ((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * v.w;
    r.y = ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * v.w;
    r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w;
    r.w = ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w;
    return r;
}

struct Corner {
    float x, y, w, cz, tx, ty, px, py, pz;
};

float edge(float ax, float ay, float bx, float by, float px, float py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

bool owns(float ax, float ay, float bx, float by) { return (ay == by && bx < ax) || by < ay; }

bool in_edge(float e, bool own) { return e > 0.0f || (e == 0.0f && own); }

// Fragments of one particle's sprite: calls frag(pixel index, depth) for
// every fragment that survives clipping and the disc test (depth unused for
// the thickness pass).
template <class F>
void sprite(int pass, const float* x4, const float* V, const float* P, uint32_t W, uint32_t H,
            F&& frag) {
    const V4 c{0.2f * x4[0] + 0.2f * -64.0f, 0.2f * x4[1] + 0.2f * 1.0f, 0.2f * x4[2] + 0.2f * -64.0f,
               1.0f};
    const V4 m = mul4(V, c);
    const float ow = pass == 0 ? 1.0f : 0.1f;
    const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
    const float cvx[4] = {-1.0f, 1.0f, 1.0f, -1.0f}, cvy[4] = {1.0f, 1.0f, -1.0f, -1.0f};
    Corner q[4];
    int near_out = 0, far_out = 0;
    float xmin = 3.0e38f, xmax = -3.0e38f, ymin = 3.0e38f, ymax = -3.0e38f;
    for (int k = 0; k < 4; ++k) {
        const V4 ps{m.x + 0.1f * cvx[k], m.y + 0.1f * cvy[k], m.z + 0.0f, m.w + ow};
        const V4 cl = mul4(P, ps);
        if (!(cl.w > 0.0f)) return;
        near_out += cl.z < -cl.w;
        far_out += cl.z > cl.w;
        q[k] = Corner{hw * (cl.x / cl.w) + hw, hh * (cl.y / cl.w) + hh, cl.w, cl.z, cvx[k], cvy[k],
                      ps.x, ps.y, ps.z};
        xmin = std::fmin(xmin, q[k].x);
        xmax = std::fmax(xmax, q[k].x);
        ymin = std::fmin(ymin, q[k].y);
        ymax = std::fmax(ymax, q[k].y);
    }
    if (near_out == 4 || far_out == 4) return;
    const bool clip_depth = near_out > 0 || far_out > 0;
    const float fx0 = std::ceil(xmin - 0.5f), fx1 = std::floor(xmax - 0.5f);
    const float fy0 = std::ceil(ymin - 0.5f), fy1 = std::floor(ymax - 0.5f);
    if (!(fx0 <= fx1) || !(fy0 <= fy1)) return;
    if (fx1 < 0.0f || fy1 < 0.0f || fx0 >= (float)W || fy0 >= (float)H) return;
    const int x0 = (int)std::fmax(fx0, 0.0f), x1 = (int)std::fmin(fx1, (float)W - 1.0f);
    const int y0 = (int)std::fmax(fy0, 0.0f), y1 = (int)std::fmin(fy1, (float)H - 1.0f);
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
                const Corner &a = q[i0], &b = q[i1], &cc = q[i2];
                const float e0 = edge(b.x, b.y, cc.x, cc.y, px, py);
                const float e1 = edge(cc.x, cc.y, a.x, a.y, px, py);
                const float e2 = edge(a.x, a.y, b.x, b.y, px, py);
                if (!in_edge(e0, owns(b.x, b.y, cc.x, cc.y)) || !in_edge(e1, owns(cc.x, cc.y, a.x, a.y)) ||
                    !in_edge(e2, owns(a.x, a.y, b.x, b.y)))
                    continue;
                const float l0 = (e0 / area) / a.w, l1 = (e1 / area) / b.w, l2 = (e2 / area) / cc.w;
                const float ls = (l0 + l1) + l2;
                auto interp = [&](float A, float B, float C) { return ((l0 * A + l1 * B) + l2 * C) / ls; };
                if (clip_depth) {
                    const float zc = interp(a.cz, b.cz, cc.cz), wc = interp(a.w, b.w, cc.w);
                    if (zc < -wc || zc > wc) break;
                }
                const float u = interp(a.tx, b.tx, cc.tx), v = interp(a.ty, b.ty, cc.ty);
                const float r = u * u + v * v;
                if (r > 1.0f) break;
                const size_t pix = (size_t)ty * W + tx;
                if (pass != 0) {
                    frag(pix, 0.0f);
                } else {
                    const float nz = -std::sqrt(1.0f - r);
                    const V4 fp{interp(a.px, b.px, cc.px) - 0.1f * u, interp(a.py, b.py, cc.py) - 0.1f * v,
                                interp(a.pz, b.pz, cc.pz) - 0.1f * nz, 1.0f};
                    const V4 cp = mul4(P, fp);
                    float d = cp.z / cp.w;
                    if (d != d) break;
                    d = d < 0.0f ? 0.0f : (d > 1.0f ? 1.0f : d);
                    frag(pix, d);
                }
                break;
            }
        }
    }
}

}  // namespace

extern "C" {

// pass 0 = depth, 1 = thickness; x4: float4[n]; V, P: column-major 4x4;
// out: float[H][W].
void pbfo_splat(int pass, const float* x4, uint32_t n, const float* V, const float* P, uint32_t W,
                uint32_t H, float* out) {
    const size_t count = (size_t)W * H;
    for (size_t k = 0; k < count; ++k) out[k] = pass == 0 ? 1.0f : 0.0f;
    for (uint32_t i = 0; i < n; ++i)
        sprite(pass, x4 + 4 * (size_t)i, V, P, W, H, [&](size_t pix, float d) {
            if (pass == 0) {
                if (d < out[pix]) out[pix] = d;
            } else {
                out[pix] += 1.0f;
            }
        });
}

}  // extern "C"
