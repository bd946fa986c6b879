// ref_shim.h -- TEST INFRASTRUCTURE ONLY.
//
// Just enough of GLSL 4.50 semantics, in C++20, to compile the reference's
// own shaders (Twinklebear/webgpu-bcmc shaders/*.comp and the isosurface
// vertex/fragment shaders, after the mechanical rewrites in ref_build.py) as
// host code, so that the CPU oracle can be checked against the reference's
// shader source itself.
//
// Semantics chosen to match how the reference runs (GLSL -> SPIR-V -> WGSL
// under Dawn): uint/int are 32-bit and wrap (built with -fwrapv), f32
// arithmetic is not contracted (-ffp-contract=off), float -> uint/int
// conversion saturates as WGSL's u32()/i32() do, min/max follow the GLSL
// definitions, and barrier() is a workgroup barrier implemented with fibers
// by ref_runtime.cpp.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <type_traits>

typedef uint32_t uint;

namespace glsl {

template <class To, class From>
inline To cvt(From f)
{
    if constexpr (std::is_floating_point_v<From> && std::is_integral_v<To> && !std::is_same_v<To, bool>) {
        // WGSL u32()/i32(): saturating, NaN -> 0
        if (f != f) return To(0);
        const double lo = (double)std::numeric_limits<To>::min(), hi = (double)std::numeric_limits<To>::max();
        const double d = (double)f;
        if (d <= lo) return std::numeric_limits<To>::min();
        if (d >= hi) return std::numeric_limits<To>::max();
        return (To)d;
    } else {
        return static_cast<To>(f);
    }
}

template <class T, int N>
struct VS;
template <class T>
struct VS<T, 2> {
    T x, y;
};
template <class T>
struct VS<T, 3> {
    T x, y, z;
};
template <class T>
struct VS<T, 4> {
    T x, y, z, w;
};

template <class T, int N>
struct V : VS<T, N> {
    V() : VS<T, N>{} {}
    template <class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>
    explicit V(S s)
    {
        for (int i = 0; i < N; ++i) (*this)[i] = cvt<T>(s);
    }
    template <class A, class B>
    V(A a, B b)
        requires(N == 2)
    {
        this->x = cvt<T>(a);
        this->y = cvt<T>(b);
    }
    template <class A, class B, class C>
    V(A a, B b, C c)
        requires(N == 3)
    {
        this->x = cvt<T>(a);
        this->y = cvt<T>(b);
        (*this)[2] = cvt<T>(c);
    }
    template <class A, class B, class C, class D>
    V(A a, B b, C c, D d)
        requires(N == 4)
    {
        this->x = cvt<T>(a);
        this->y = cvt<T>(b);
        (*this)[2] = cvt<T>(c);
        (*this)[3] = cvt<T>(d);
    }
    template <class U, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>
    V(const V<U, 3>& a, S s)
        requires(N == 4)
    {
        this->x = cvt<T>(a[0]);
        this->y = cvt<T>(a[1]);
        (*this)[2] = cvt<T>(a[2]);
        (*this)[3] = cvt<T>(s);
    }
    // GLSL's implicit int -> uint -> float conversions between vector types
    template <class U, class = std::enable_if_t<!std::is_same_v<U, T>>>
    V(const V<U, N>& o)
    {
        for (int i = 0; i < N; ++i) (*this)[i] = cvt<T>(o[i]);
    }
    T& operator[](int i) { return (&this->x)[i]; }
    const T& operator[](int i) const { return (&this->x)[i]; }
    T& operator[](uint i) { return (&this->x)[i]; }
    const T& operator[](uint i) const { return (&this->x)[i]; }
};

template <class A, class B>
using common_t = std::common_type_t<A, B>;

#define GLSL_VEC_BINOP(OP)                                                                         \
    template <class A, class B, int N>                                                             \
    inline V<common_t<A, B>, N> operator OP(const V<A, N>& a, const V<B, N>& b)                    \
    {                                                                                              \
        V<common_t<A, B>, N> r;                                                                    \
        for (int i = 0; i < N; ++i) r[i] = (common_t<A, B>)a[i] OP(common_t<A, B>) b[i];           \
        return r;                                                                                  \
    }                                                                                              \
    template <class A, class S, int N, class = std::enable_if_t<std::is_arithmetic_v<S>>>          \
    inline V<common_t<A, S>, N> operator OP(const V<A, N>& a, S s)                                 \
    {                                                                                              \
        V<common_t<A, S>, N> r;                                                                    \
        for (int i = 0; i < N; ++i) r[i] = (common_t<A, S>)a[i] OP(common_t<A, S>) s;              \
        return r;                                                                                  \
    }                                                                                              \
    template <class A, class S, int N, class = std::enable_if_t<std::is_arithmetic_v<S>>>          \
    inline V<common_t<A, S>, N> operator OP(S s, const V<A, N>& a)                                 \
    {                                                                                              \
        V<common_t<A, S>, N> r;                                                                    \
        for (int i = 0; i < N; ++i) r[i] = (common_t<A, S>)s OP(common_t<A, S>) a[i];              \
        return r;                                                                                  \
    }
GLSL_VEC_BINOP(+)
GLSL_VEC_BINOP(-)
GLSL_VEC_BINOP(*)
GLSL_VEC_BINOP(/)
GLSL_VEC_BINOP(%)
#undef GLSL_VEC_BINOP

template <class A, class B, int N>
inline V<A, N>& operator+=(V<A, N>& a, const B& b)
{
    a = V<A, N>(a + b);
    return a;
}
template <class A, class B, int N>
inline V<A, N>& operator-=(V<A, N>& a, const B& b)
{
    a = V<A, N>(a - b);
    return a;
}

// GLSL == / != on vectors compare all components and return bool
template <class A, class B, int N>
inline bool operator==(const V<A, N>& a, const V<B, N>& b)
{
    for (int i = 0; i < N; ++i)
        if ((common_t<A, B>)a[i] != (common_t<A, B>)b[i]) return false;
    return true;
}
template <class A, class B, int N>
inline bool operator!=(const V<A, N>& a, const V<B, N>& b)
{
    return !(a == b);
}

#define GLSL_VEC_CMP(NAME, OP)                                                                     \
    template <class A, class B, int N>                                                             \
    inline V<bool, N> NAME(const V<A, N>& a, const V<B, N>& b)                                     \
    {                                                                                              \
        V<bool, N> r;                                                                              \
        for (int i = 0; i < N; ++i) r[i] = (common_t<A, B>)a[i] OP(common_t<A, B>) b[i];           \
        return r;                                                                                  \
    }
GLSL_VEC_CMP(lessThan, <)
GLSL_VEC_CMP(lessThanEqual, <=)
GLSL_VEC_CMP(greaterThan, >)
GLSL_VEC_CMP(greaterThanEqual, >=)
#undef GLSL_VEC_CMP

template <int N>
inline bool any(const V<bool, N>& b)
{
    for (int i = 0; i < N; ++i)
        if (b[i]) return true;
    return false;
}
template <int N>
inline bool all(const V<bool, N>& b)
{
    for (int i = 0; i < N; ++i)
        if (!b[i]) return false;
    return true;
}

// Swizzles used by the shaders: .xyz reads, .xy/.xz/.yz read, compare and assign.
template <class Vec>
inline auto swz_xyz(const Vec& v)
{
    return V<std::remove_cv_t<std::remove_reference_t<decltype(v[0])>>, 3>(v[0], v[1], v[2]);
}
// `v.xyz = e` (the target of an assignment)
template <class Vec>
struct SetXyz {
    Vec& v;
    template <class U>
    SetXyz& operator=(const V<U, 3>& o)
    {
        using T = std::remove_cv_t<std::remove_reference_t<decltype(v[0])>>;
        v[0] = cvt<T>(o[0]);
        v[1] = cvt<T>(o[1]);
        v[2] = cvt<T>(o[2]);
        return *this;
    }
};
template <class Vec>
inline SetXyz<Vec> set_xyz(Vec& v)
{
    return {v};
}

// mat4: four vec4 columns; m * v = sum_i m[i] * v[i], added in column order
struct mat4 {
    V<float, 4> c[4];
    V<float, 4>& operator[](int i) { return c[i]; }
    const V<float, 4>& operator[](int i) const { return c[i]; }
};
inline V<float, 4> operator*(const mat4& m, const V<float, 4>& v)
{
    V<float, 4> r;
    for (int row = 0; row < 4; ++row) {
        float acc = m.c[0][row] * v[0];
        for (int i = 1; i < 4; ++i) acc = acc + m.c[i][row] * v[i];
        r[row] = acc;
    }
    return r;
}

template <class Vec, int I, int J>
struct Swz2 {
    Vec& v;
    using T = std::remove_cv_t<std::remove_reference_t<decltype(v[0])>>;
    operator V<T, 2>() const { return V<T, 2>(v[I], v[J]); }
    template <class U>
    Swz2& operator=(const V<U, 2>& o)
    {
        v[I] = cvt<T>(o[0]);
        v[J] = cvt<T>(o[1]);
        return *this;
    }
    template <class U>
    bool operator==(const V<U, 2>& o) const
    {
        return V<T, 2>(v[I], v[J]) == o;
    }
};
template <class Vec>
inline Swz2<Vec, 0, 1> swz_xy(Vec& v)
{
    return {v};
}
template <class Vec>
inline Swz2<Vec, 0, 2> swz_xz(Vec& v)
{
    return {v};
}
template <class Vec>
inline Swz2<Vec, 1, 2> swz_yz(Vec& v)
{
    return {v};
}

template <class T, int N>
inline V<T, N> operator-(const V<T, N>& a)
{
    V<T, N> r;
    for (int i = 0; i < N; ++i) r[i] = -a[i];
    return r;
}

// GLSL min/max definitions: min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x
template <class T>
inline T min(T x, T y)
{
    return y < x ? y : x;
}
template <class T>
inline T max(T x, T y)
{
    return x < y ? y : x;
}

}  // namespace glsl

// min/max/abs/ldexp calls in the shader text are renamed to these (ref_build.py)
// so that they cannot collide with the C library's overloads.
template <class T>
inline T glsl_min(T x, T y)
{
    return glsl::min(x, y);
}
template <class T>
inline T glsl_max(T x, T y)
{
    return glsl::max(x, y);
}
inline float glsl_abs(float x) { return std::fabs(x); }
inline int glsl_abs(int x) { return x < 0 ? -x : x; }
inline float glsl_ldexp(float x, int e) { return std::ldexp(x, e); }
inline float glsl_ceil(float x) { return std::ceil(x); }
inline float glsl_max(float x, int y) { return glsl::max(x, (float)y); }
template <class T, int N>
inline glsl::V<T, N> glsl_min(const glsl::V<T, N>& x, const glsl::V<T, N>& y)
{
    glsl::V<T, N> r;
    for (int i = 0; i < N; ++i) r[i] = glsl::min(x[i], y[i]);
    return r;
}
template <class T, int N>
inline glsl::V<T, N> glsl_max(const glsl::V<T, N>& x, const glsl::V<T, N>& y)
{
    glsl::V<T, N> r;
    for (int i = 0; i < N; ++i) r[i] = glsl::max(x[i], y[i]);
    return r;
}

using glsl::all;
using glsl::any;
using glsl::greaterThan;
using glsl::greaterThanEqual;
using glsl::lessThan;
using glsl::lessThanEqual;

typedef glsl::V<float, 2> vec2;
typedef glsl::V<float, 3> vec3;
typedef glsl::V<float, 4> vec4;
typedef glsl::V<int, 2> ivec2;
typedef glsl::V<int, 3> ivec3;
typedef glsl::V<int, 4> ivec4;
typedef glsl::V<uint, 2> uvec2;
typedef glsl::V<uint, 3> uvec3;
typedef glsl::V<uint, 4> uvec4;
typedef glsl::V<bool, 3> bvec3;
typedef glsl::mat4 mat4;

// vertex-stage built-in output
extern vec4 gl_Position;

// Geometric and exponential built-ins of the isosurface shaders, by their GLSL
// definitions: dot sums the products in component order, length(x) =
// sqrt(dot(x, x)), normalize(x) = x / length(x), clamp(x, a, b) =
// min(max(x, a), b).
inline float glsl_dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float glsl_length(const vec3& a) { return std::sqrt(glsl_dot(a, a)); }
inline vec3 glsl_normalize(const vec3& a)
{
    const float l = glsl_length(a);
    return vec3(a.x / l, a.y / l, a.z / l);
}
inline vec3 glsl_cross(const vec3& a, const vec3& b)
{
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float glsl_clamp(float x, float lo, float hi) { return glsl::min(glsl::max(x, lo), hi); }
inline float glsl_pow(float x, float y) { return std::pow(x, y); }
inline float glsl_exp(float x) { return std::exp(x); }
// Screen-space derivatives of the fragment's world position: the harness sets
// them for the fragment being shaded (one fragment runs at a time).
extern vec3 ref_dfdx, ref_dfdy;
inline vec3 glsl_dFdx(const vec3&) { return ref_dfdx; }
inline vec3 glsl_dFdy(const vec3&) { return ref_dfdy; }

// Invocation ids of the running invocation (set by the runtime before it
// resumes each invocation) and the workgroup barrier.
extern uvec3 gl_GlobalInvocationID;
extern uvec3 gl_LocalInvocationID;
extern uvec3 gl_WorkGroupID;
void ref_barrier();

// Runs `invocations` invocations of `main_fn` per workgroup over `groups`
// workgroups (x-major ids), as fibers that switch at barrier().
void ref_dispatch(void (*main_fn)(), uvec3 groups, uint invocations);

// The same for programs that call no barrier() and share no workgroup memory:
// invocations run one after another in id order, without fibers.  A barrier()
// reached in this mode aborts the process.
void ref_dispatch_flat(void (*main_fn)(), uvec3 groups, uint invocations);
