// Minimal, from-scratch subset of the glm vector/matrix API.
//
// Test infrastructure only: it exists so that the reference solver's own
// physics sources (which include <glm/glm.hpp> and "./include/glm/glm.hpp",
// a header-only library that the reference does not vendor) can be compiled
// headless as the parity oracle.  Nothing in the product links it.
//
// Semantics follow glm's published documentation: column-major matrices
// (m[c] is column c, m[c][r] is the element in row r), component-wise vector
// arithmetic, and the classic cofactor formula for the 3x3 determinant.  The
// exact operation order chosen here for dot/length/normalize, mat*mat,
// mat*vec, determinant and outerProduct is written down in this file and is
// mirrored by the CPU restatement (oracle/mpm_oracle.c) and the CUDA kernels;
// no pinned glm release exists to compare it against.
#ifndef MPM_GLMSHIM_GLM_HPP
#define MPM_GLMSHIM_GLM_HPP

#include <array>
#include <cmath>
#include <cstddef>
#include <type_traits>

namespace glm {

template <int L, typename T> struct vec;

template <typename T> struct vec<2, T> {
    T x, y;
    vec() : x(0), y(0) {}
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    explicit vec(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)) {}
    template <typename A, typename B>
    vec(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    template <typename U> vec(const vec<2, U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}
    // the first two components of a longer vector (glm's explicit truncation)
    template <int L, typename U, typename = typename std::enable_if<(L > 2)>::type>
    explicit vec(const vec<L, U>& o) : x(static_cast<T>(o[0])), y(static_cast<T>(o[1])) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    static constexpr int length() { return 2; }
};

template <typename T> struct vec<3, T> {
    T x, y, z;
    vec() : x(0), y(0), z(0) {}
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    explicit vec(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)) {}
    template <typename A, typename B, typename C>
    vec(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U, typename C>
    vec(const vec<2, U>& xy, C c) : x(static_cast<T>(xy.x)), y(static_cast<T>(xy.y)), z(static_cast<T>(c)) {}
    template <typename U>
    vec(const vec<3, U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    static constexpr int length() { return 3; }
};

template <typename T> struct vec<4, T>;

template <typename T> struct vec<4, T> {
    T x, y, z, w;
    vec() : x(0), y(0), z(0), w(0) {}
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    explicit vec(S s) : x(static_cast<T>(s)), y(static_cast<T>(s)), z(static_cast<T>(s)), w(static_cast<T>(s)) {}
    template <typename A, typename B, typename C, typename D>
    vec(A a, B b, C c, D d)
        : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
    template <typename U, typename D>
    vec(const vec<3, U>& v, D d) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(d)) {}
    template <typename U, typename C, typename D>
    vec(const vec<2, U>& v, C c, D d)
        : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
    template <typename U>
    vec(const vec<4, U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)), w(static_cast<T>(o.w)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    static constexpr int length() { return 4; }
};

typedef vec<2, float> vec2;
typedef vec<3, float> vec3;
typedef vec<4, float> vec4;
typedef vec<2, double> dvec2;
typedef vec<3, double> dvec3;
typedef vec<4, double> dvec4;
typedef vec<2, int> ivec2;
typedef vec<3, int> ivec3;
typedef vec<4, int> ivec4;
typedef vec<2, unsigned int> uvec2;
typedef vec<3, unsigned int> uvec3;
typedef vec<2, bool> bvec2;
typedef vec<3, bool> bvec3;

// ---- component-wise arithmetic -------------------------------------------
#define MPM_GLMSHIM_BINOP(OP)                                                              \
    template <int L, typename T> vec<L, T> operator OP(const vec<L, T>& a, const vec<L, T>& b) { \
        vec<L, T> r;                                                                        \
        for (int i = 0; i < L; ++i) r[i] = a[i] OP b[i];                                    \
        return r;                                                                           \
    }                                                                                       \
    template <int L, typename T, typename S,                                                \
              typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>       \
    vec<L, T> operator OP(const vec<L, T>& a, S s) {                                        \
        vec<L, T> r;                                                                        \
        for (int i = 0; i < L; ++i) r[i] = a[i] OP static_cast<T>(s);                       \
        return r;                                                                           \
    }                                                                                       \
    template <int L, typename T, typename S,                                                \
              typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>       \
    vec<L, T> operator OP(S s, const vec<L, T>& a) {                                        \
        vec<L, T> r;                                                                        \
        for (int i = 0; i < L; ++i) r[i] = static_cast<T>(s) OP a[i];                       \
        return r;                                                                           \
    }                                                                                       \
    template <int L, typename T> vec<L, T>& operator OP##=(vec<L, T>& a, const vec<L, T>& b) { \
        for (int i = 0; i < L; ++i) a[i] = a[i] OP b[i];                                    \
        return a;                                                                           \
    }                                                                                       \
    template <int L, typename T, typename S,                                                \
              typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>       \
    vec<L, T>& operator OP##=(vec<L, T>& a, S s) {                                          \
        for (int i = 0; i < L; ++i) a[i] = a[i] OP static_cast<T>(s);                       \
        return a;                                                                           \
    }
MPM_GLMSHIM_BINOP(+)
MPM_GLMSHIM_BINOP(-)
MPM_GLMSHIM_BINOP(*)
MPM_GLMSHIM_BINOP(/)
#undef MPM_GLMSHIM_BINOP

template <int L, typename T> vec<L, T> operator-(const vec<L, T>& a) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = -a[i];
    return r;
}
template <int L, typename T> bool operator==(const vec<L, T>& a, const vec<L, T>& b) {
    for (int i = 0; i < L; ++i)
        if (!(a[i] == b[i])) return false;
    return true;
}
template <int L, typename T> bool operator!=(const vec<L, T>& a, const vec<L, T>& b) { return !(a == b); }

// ---- scalar functions ----------------------------------------------------
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T abs(T x) { return x >= T(0) ? x : -x; }
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T sign(T x) { return static_cast<T>((T(0) < x) - (x < T(0))); }
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T max(T a, T b) { return (a < b) ? b : a; }
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T min(T a, T b) { return (b < a) ? b : a; }
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
inline double sqrt(double x) { return std::sqrt(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline double pow(double a, double b) { return std::pow(a, b); }
inline double pow(double a, int b) { return std::pow(a, static_cast<double>(b)); }
inline double cos(double x) { return std::cos(x); }
inline double sin(double x) { return std::sin(x); }
inline double acos(double x) { return std::acos(x); }
inline double floor(double x) { return std::floor(x); }
inline double radians(double d) { return d * 0.01745329251994329576923690768489; }

// ---- vector functions ----------------------------------------------------
template <int L, typename T> vec<L, T> abs(const vec<L, T>& a) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = glm::abs(a[i]);
    return r;
}
template <int L, typename T> vec<L, T> sign(const vec<L, T>& a) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = glm::sign(a[i]);
    return r;
}
template <int L, typename T> vec<L, T> floor(const vec<L, T>& a) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = std::floor(a[i]);
    return r;
}
template <int L, typename T> vec<L, T> sqrt(const vec<L, T>& a) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = std::sqrt(a[i]);
    return r;
}
template <int L, typename T> vec<L, T> max(const vec<L, T>& a, const vec<L, T>& b) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = glm::max(a[i], b[i]);
    return r;
}
template <int L, typename T> vec<L, T> min(const vec<L, T>& a, const vec<L, T>& b) {
    vec<L, T> r;
    for (int i = 0; i < L; ++i) r[i] = glm::min(a[i], b[i]);
    return r;
}
// dot: products formed first, then summed left to right.
template <int L, typename T> T dot(const vec<L, T>& a, const vec<L, T>& b) {
    T s = a[0] * b[0];
    for (int i = 1; i < L; ++i) s = s + a[i] * b[i];
    return s;
}
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T dot(T a, T b) { return a * b; }
template <int L, typename T> T length(const vec<L, T>& a) { return std::sqrt(dot(a, a)); }
template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
T length(T a) { return glm::abs(a); }
template <int L, typename T> T distance(const vec<L, T>& a, const vec<L, T>& b) { return length(b - a); }
template <int L, typename T> vec<L, T> normalize(const vec<L, T>& a) {
    return a * (T(1) / std::sqrt(dot(a, a)));
}
template <typename T> vec<3, T> cross(const vec<3, T>& a, const vec<3, T>& b) {
    return vec<3, T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ---- 3x3 matrix (column-major) -------------------------------------------
template <typename T> struct mat3x3 {
    vec<3, T> c[3];
    mat3x3() { *this = mat3x3(T(1)); }
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    explicit mat3x3(S s) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) c[i][j] = (i == j) ? static_cast<T>(s) : T(0);
    }
    mat3x3(const vec<3, T>& c0, const vec<3, T>& c1, const vec<3, T>& c2) { c[0] = c0; c[1] = c1; c[2] = c2; }
    vec<3, T>& operator[](int i) { return c[i]; }
    const vec<3, T>& operator[](int i) const { return c[i]; }
    mat3x3& operator+=(const mat3x3& o) { for (int i = 0; i < 3; ++i) c[i] += o.c[i]; return *this; }
    mat3x3& operator-=(const mat3x3& o) { for (int i = 0; i < 3; ++i) c[i] -= o.c[i]; return *this; }
    mat3x3& operator*=(const mat3x3& o);
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    mat3x3& operator*=(S s) { for (int i = 0; i < 3; ++i) c[i] *= s; return *this; }
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    mat3x3& operator/=(S s) { for (int i = 0; i < 3; ++i) c[i] /= s; return *this; }
};
typedef mat3x3<double> dmat3;
typedef mat3x3<float> mat3;

template <typename T> mat3x3<T> operator+(const mat3x3<T>& a, const mat3x3<T>& b) {
    return mat3x3<T>(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
}
template <typename T> mat3x3<T> operator-(const mat3x3<T>& a, const mat3x3<T>& b) {
    return mat3x3<T>(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
template <typename T, typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
mat3x3<T> operator*(const mat3x3<T>& a, S s) { return mat3x3<T>(a[0] * s, a[1] * s, a[2] * s); }
template <typename T, typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
mat3x3<T> operator*(S s, const mat3x3<T>& a) { return mat3x3<T>(s * a[0], s * a[1], s * a[2]); }
template <typename T, typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
mat3x3<T> operator/(const mat3x3<T>& a, S s) { return mat3x3<T>(a[0] / s, a[1] / s, a[2] / s); }
// (A*B)[c][r] = (A[0][r]*B[c][0] + A[1][r]*B[c][1]) + A[2][r]*B[c][2]
template <typename T> mat3x3<T> operator*(const mat3x3<T>& a, const mat3x3<T>& b) {
    mat3x3<T> r(T(0));
    for (int col = 0; col < 3; ++col)
        for (int row = 0; row < 3; ++row)
            r[col][row] = a[0][row] * b[col][0] + a[1][row] * b[col][1] + a[2][row] * b[col][2];
    return r;
}
// (M*v)[r] = (M[0][r]*v.x + M[1][r]*v.y) + M[2][r]*v.z
template <typename T> vec<3, T> operator*(const mat3x3<T>& m, const vec<3, T>& v) {
    return vec<3, T>(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z,
                     m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
                     m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z);
}
template <typename T> mat3x3<T>& mat3x3<T>::operator*=(const mat3x3<T>& o) { return (*this = *this * o); }

template <typename T> mat3x3<T> transpose(const mat3x3<T>& m) {
    mat3x3<T> r(T(0));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i][j] = m[j][i];
    return r;
}
// Cofactor expansion along the first row of the column-major storage.
template <typename T> T determinant(const mat3x3<T>& m) {
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2])
         - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2])
         + m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}
// outerProduct(c, r)[i][j] = c[j] * r[i]  (column i, row j)
template <typename T> mat3x3<T> outerProduct(const vec<3, T>& c, const vec<3, T>& r) {
    mat3x3<T> m(T(0));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m[i][j] = c[j] * r[i];
    return m;
}

// ---- 4x4 matrix (column-major), for the canvas transforms ------------------
template <typename T> struct mat4x4 {
    vec<4, T> c[4];
    mat4x4() { *this = mat4x4(T(1)); }
    template <typename S, typename = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    explicit mat4x4(S s) {
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) c[i][j] = (i == j) ? static_cast<T>(s) : T(0);
    }
    vec<4, T>& operator[](int i) { return c[i]; }
    const vec<4, T>& operator[](int i) const { return c[i]; }
    mat4x4& operator*=(const mat4x4& o);
};
typedef mat4x4<double> dmat4;
typedef mat4x4<float> mat4;

// (A*B)[c][r] = ((A[0][r]*B[c][0] + A[1][r]*B[c][1]) + A[2][r]*B[c][2]) + A[3][r]*B[c][3]
template <typename T> mat4x4<T> operator*(const mat4x4<T>& a, const mat4x4<T>& b) {
    mat4x4<T> r(T(0));
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row)
            r[col][row] = a[0][row] * b[col][0] + a[1][row] * b[col][1] + a[2][row] * b[col][2] + a[3][row] * b[col][3];
    return r;
}
template <typename T> mat4x4<T>& mat4x4<T>::operator*=(const mat4x4<T>& o) { return (*this = *this * o); }
// (M*v)[r] = ((M[0][r]*v.x + M[1][r]*v.y) + M[2][r]*v.z) + M[3][r]*v.w
template <typename T> vec<4, T> operator*(const mat4x4<T>& m, const vec<4, T>& v) {
    vec<4, T> r;
    for (int row = 0; row < 4; ++row) r[row] = m[0][row] * v.x + m[1][row] * v.y + m[2][row] * v.z + m[3][row] * v.w;
    return r;
}
// translation by v: the identity with v in the last column
template <typename T> mat4x4<T> translate(const vec<3, T>& v) {
    mat4x4<T> m(T(1));
    m[3][0] = v.x;
    m[3][1] = v.y;
    m[3][2] = v.z;
    return m;
}
// rotation by `angle` (radians) about the unit vector along `axis`:
// R = cos(a) I + (1 - cos(a)) n n^T + sin(a) [n]x (Rodrigues' formula)
template <typename T> mat4x4<T> rotate(T angle, const vec<3, T>& axis) {
    const T cs = std::cos(angle), sn = std::sin(angle);
    const vec<3, T> n = normalize(axis);
    mat4x4<T> m(T(1));
    const T k[3][3] = {{T(0), -n.z, n.y}, {n.z, T(0), -n.x}, {-n.y, n.x, T(0)}};  // [n]x by row
    for (int col = 0; col < 3; ++col)
        for (int row = 0; row < 3; ++row)
            m[col][row] = (col == row ? cs : T(0)) + (T(1) - cs) * n[row] * n[col] + sn * k[row][col];
    return m;
}

}  // namespace glm

#endif  // MPM_GLMSHIM_GLM_HPP
