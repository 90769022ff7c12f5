// glsl.hpp — the slice of GLSL 4.30 the reference's compute shaders use,
// as C++, so that their source compiles on the CPU (TEST INFRASTRUCTURE:
// the reference-pinning recipe, oracle/ref_build.py).
//
// Arithmetic follows the shaders literally: one rounding per operation, in
// the order written (compile with -ffp-contract=off), float literals as
// float (-fsingle-precision-constant), sqrt correctly rounded.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

static_assert(sizeof(float) == 4, "float");

namespace glsl {

typedef unsigned int uint;

struct vec2;
struct vec3;
struct ivec3;

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
};
inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }


// .xyz of a 3- or 4-vector: storage shared with the vector's lanes
template <typename T, typename V3, int N>
struct Swizzle3 {
    T v[N];
    operator V3() const { return V3(v[0], v[1], v[2]); }
};

struct vec3 {
    union {
        struct {
            float x, y, z;
        };
        Swizzle3<float, vec3, 3> xyz;
    };
    vec3() : x(0), y(0), z(0) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    vec3& operator=(const vec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        return *this;
    }
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(vec2 a, float c) : x(a.x), y(a.y), z(c) {}
    explicit vec3(float a) : x(a), y(a), z(a) {}
    explicit vec3(const ivec3& v);
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator-=(const vec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    vec3& operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
    vec3& operator/=(float s) { x = x / s; y = y / s; z = z / s; return *this; }
};

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
// int * vec3 (e.g. 2 * gravity * vec3(...)) promotes the int to float
inline vec3 operator*(int s, vec3 a) { return float(s) * a; }

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    // GLSL int(float) truncates toward zero
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
    int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline vec3::vec3(const ivec3& v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
inline ivec3 operator+(ivec3 a, ivec3 b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator*(int s, ivec3 a) { return ivec3(s * a.x, s * a.y, s * a.z); }
inline bool operator==(ivec3 a, ivec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(ivec3 a, ivec3 b) { return !(a == b); }


struct vec4 {
    union {
        struct {
            float x, y, z, w;
        };
        Swizzle3<float, vec3, 4> xyz;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(vec2 v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
};
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

// mat4: four columns; mat4 * vec4 sums the column terms left to right.
struct mat4 {
    vec4 c[4];
};
inline vec4 operator*(const mat4& m, vec4 v) {
    return vec4(((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z) + m.c[3].x * v.w,
                ((m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z) + m.c[3].y * v.w,
                ((m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z) + m.c[3].z * v.w,
                ((m.c[0].w * v.x + m.c[1].w * v.y) + m.c[2].w * v.z) + m.c[3].w * v.w);
}

struct ivec4 {
    union {
        struct {
            int x, y, z, w;
        };
        Swizzle3<int, ivec3, 4> xyz;
    };
    ivec4() : x(0), y(0), z(0), w(0) {}
    ivec4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
};

struct uvec3 {
    uint x, y, z;
};
struct uvec4 {
    uint x, y, z, w;
};

inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// GLSL has no integer dot: ivec3 arguments convert to vec3 implicitly, so
// GetHash (counting.glsl:56) computes the key in float (exact below 2^24).
inline float dot(ivec3 a, ivec3 b) { return dot(vec3(a), vec3(b)); }
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline float sqrt(float a) { return std::sqrt(a); }
inline float distance(vec3 a, vec3 b) { return length(a - b); }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float clampf(float v, float lo, float hi) { return std::fmin(std::fmax(v, lo), hi); }
inline vec3 clamp(vec3 v, vec3 lo, vec3 hi) {
    return vec3(clampf(v.x, lo.x, hi.x), clampf(v.y, lo.y, hi.y), clampf(v.z, lo.z, hi.z));
}
inline int floatBitsToInt(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline float intBitsToFloat(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

// ---- textures and images --------------------------------------------------------

struct samplerBuffer {  // rgba32f (4 lanes) or r32f (1 lane)
    const float* data = nullptr;
    int lanes = 4;
};
struct isamplerBuffer {  // rgba32i
    const int* data = nullptr;
};
struct isampler3D {  // r32i, dims; outside the grid reads the border -1
    const int* data = nullptr;
    int dx = 0, dy = 0, dz = 0;
};
struct sampler3D {};
struct imageBuffer {  // rgba32f or r32f
    float* data = nullptr;
    int lanes = 4;
};
struct iimage3D {
    int* data = nullptr;
    int dx = 0, dy = 0, dz = 0;
};
struct iimageBuffer {
    int* data = nullptr;
};

struct uimageBuffer {  // r32ui
    uint* data = nullptr;
};

inline vec4 texelFetch(const samplerBuffer& t, int i) {
    if (t.lanes == 1) return vec4(t.data[i], 0.0f, 0.0f, 1.0f);
    return vec4(t.data[4 * i], t.data[4 * i + 1], t.data[4 * i + 2], t.data[4 * i + 3]);
}
inline ivec4 texelFetch(const isamplerBuffer& t, int i) {
    return ivec4(t.data[4 * i], t.data[4 * i + 1], t.data[4 * i + 2], t.data[4 * i + 3]);
}
inline ivec4 texelFetch(const isampler3D& t, ivec3 p, int) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= t.dx || p.y >= t.dy || p.z >= t.dz)
        return ivec4(-1, 0, 0, 1);
    return ivec4(t.data[(p.z * t.dy + p.y) * t.dx + p.x], 0, 0, 1);
}
inline vec4 imageLoad(const imageBuffer& im, int i) {
    if (im.lanes == 1) return vec4(im.data[i], 0.0f, 0.0f, 1.0f);
    return vec4(im.data[4 * i], im.data[4 * i + 1], im.data[4 * i + 2], im.data[4 * i + 3]);
}
inline void imageStore(imageBuffer& im, int i, vec4 v) {
    if (im.lanes == 1) {
        im.data[i] = v.x;
        return;
    }
    im.data[4 * i] = v.x;
    im.data[4 * i + 1] = v.y;
    im.data[4 * i + 2] = v.z;
    im.data[4 * i + 3] = v.w;
}
inline void imageStore(iimage3D& im, ivec3 p, ivec4 v) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.dx || p.y >= im.dy || p.z >= im.dz) return;
    im.data[(p.z * im.dy + p.y) * im.dx + p.x] = v.x;
}
inline void imageStore(iimageBuffer& im, int i, ivec4 v) {
    im.data[4 * i] = v.x;
    im.data[4 * i + 1] = v.y;
    im.data[4 * i + 2] = v.z;
    im.data[4 * i + 3] = v.w;
}

inline uvec4 imageLoad(const uimageBuffer& im, int i) { return uvec4{im.data[i], 0u, 0u, 1u}; }
// invocations run one after another, so the atomics are plain read-modify-writes
inline uint imageAtomicOr(uimageBuffer& im, int i, uint v) {
    const uint old = im.data[i];
    im.data[i] = old | v;
    return old;
}
inline uint imageAtomicAnd(uimageBuffer& im, int i, uint v) {
    const uint old = im.data[i];
    im.data[i] = old & v;
    return old;
}

inline void barrier() {}
inline void memoryBarrier() {}
inline void memoryBarrierShared() {}

}  // namespace glsl
