// GLSL/HLSL built-in shim that lets the reference's bgfx compute shaders
// (natrix/core/shaders/originals/*.comp, demo/shaders/shader.Add*/Advect*.comp)
// compile unchanged as C++ on the CPU.  It is test infrastructure only: the
// oracle build compiles the reference's own kernel sources against it to pin
// the oracle restatement (oracle/oracle.c) and to write golden vectors.
//
// Semantics chosen where GLSL leaves them to the driver:
//   * mix(x, y, a)      = x + a * (y - x)       (HLSL lerp form)
//   * inversesqrt(m)    = 1 / sqrt(m)           (correctly rounded sqrt and div)
//   * clamp(x, lo, hi)  = min(max(x, lo), hi)
//   * distance(a, b)    = sqrt(dot(a - b, a - b))
//   * float -> vec2     = broadcast (HLSL), vec2 -> float = .x (HLSL truncation)
// The oracle build uses -ffp-contract=off so every product and sum rounds
// separately, as the shader text is written.
#ifndef NATRIX_GLSL_SHIM_HPP
#define NATRIX_GLSL_SHIM_HPP

#include <cmath>
#include <cstddef>

namespace glsl {

typedef unsigned int uint;

struct uvec2 {
    uint x, y;
};

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}
    explicit inline ivec2(const struct vec2& v);
};

struct uvec3 {
    uint x, y, z;
    uvec2 xy;
};

struct uvec4 {
    uint x, y, z, w;
};

struct vec2 {
    float x, y;
    vec2() : x(0.0f), y(0.0f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(const uvec2& u) : x((float)u.x), y((float)u.y) {}
    explicit vec2(const ivec2& i) : x((float)i.x), y((float)i.y) {}
    explicit vec2(const uvec3& u) : x((float)u.x), y((float)u.y) {}
    operator float() const { return x; }
    vec2& operator*=(const vec2& o) { x = x * o.x; y = y * o.y; return *this; }
    vec2& operator*=(float s) { x = x * s; y = y * s; return *this; }
};

inline ivec2::ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}

inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(float s, const vec2& a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator/(const vec2& a, float s) { return vec2(a.x / s, a.y / s); }

inline float abs(float a) { return std::fabs(a); }
inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline int clamp(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec2 clamp(const vec2& x, const vec2& lo, const vec2& hi) {
    return vec2(clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y));
}
inline vec2 ceil(const vec2& a) { return vec2(std::ceil(a.x), std::ceil(a.y)); }
inline vec2 floor(const vec2& a) { return vec2(std::floor(a.x), std::floor(a.y)); }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float distance(const vec2& a, const vec2& b) {
    vec2 d = a - b;
    return std::sqrt(dot(d, d));
}
inline float inversesqrt(float m) { return 1.0f / std::sqrt(m); }
inline vec2 mix(const vec2& a, const vec2& b, const vec2& t) {
    return vec2(a.x + t.x * (b.x - a.x), a.y + t.y * (b.y - a.y));
}
// mix(float, float, vec2): HLSL promotes the scalars, the result is a vec2.
inline vec2 mix(float a, float b, const vec2& t) { return mix(vec2(a), vec2(b), t); }

// Element reference into a vec2 buffer: reads as vec2 or (HLSL truncation)
// as float, and accepts a vec2 or a broadcast float on assignment.
struct Vec2Ref {
    float& x;
    float& y;
    explicit Vec2Ref(vec2& v) : x(v.x), y(v.y) {}
    operator vec2() const { return vec2(x, y); }
    operator float() const { return x; }
    Vec2Ref& operator=(const vec2& v) { x = v.x; y = v.y; return *this; }
    Vec2Ref& operator=(float s) { x = s; y = s; return *this; }
};
inline vec2 operator+(const Vec2Ref& a, const vec2& b) { return vec2(a) + b; }

template <class T>
struct Buf {
    T* p = nullptr;
    template <class I>
    T& operator[](I i) const { return p[(std::ptrdiff_t)i]; }
};

template <>
struct Buf<vec2> {
    vec2* p = nullptr;
    template <class I>
    Vec2Ref operator[](I i) const { return Vec2Ref(p[(std::ptrdiff_t)i]); }
};

}  // namespace glsl

// One invocation id shared by every shader; the CPU dispatcher sets it.
extern glsl::uvec3 gl_GlobalInvocationID;

#define uniform static
#define BUFFER_RO(name, type, slot) static glsl::Buf<type> name
#define BUFFER_WR(name, type, slot) static glsl::Buf<type> name
#define BUFFER_RW(name, type, slot) static glsl::Buf<type> name
#define NUM_THREADS(x, y, z)

#endif  // NATRIX_GLSL_SHIM_HPP
