// Minimal column-major vector/matrix header with the glm API subset the
// reference surfel rasteriser's CUDA sources use, so that those sources can be
// compiled unmodified as a parity and timing oracle (test infrastructure only;
// nothing in the product library includes it).
//
// Written from the documented glm semantics, not from glm's source:
//  * vecN has members x, y, z, w and operator[]; arithmetic is component-wise,
//    scalars broadcast; vec3(vec4) drops w, vec4(vec3, w) appends w.
//  * mat<C, R> ("matCxR") holds C columns of R rows; m[c] is column c, so
//    m[c][r] is the element in row r of column c.  Scalar constructors fill
//    column after column; mat(s) puts s on the diagonal.
//  * mat<C1,R1> * mat<C2,C1> -> mat<C2,R1>; mat<C,R> * vec<C> -> vec<R>
//    (column vector); vec<R> * mat<C,R> -> vec<C> (row vector).
//  * dot, length, normalize, cross, transpose, sqrt/abs as usual; max(x, y)
//    is (x < y) ? y : x and min(x, y) is (y < x) ? y : x, per component.
// Sums run in index order (k = 0, 1, ...), the textbook definition.
//
// Used by the reference's forward.cu, backward.cu, auxiliary.h and
// rasterizer_impl.cu of both rasteriser variants (types glm::vec2/3/4,
// glm::mat3, mat4, mat3x4, mat4x3; functions glm::dot, length, max, transpose,
// and sqrt/max found by argument-dependent lookup).
#pragma once

#include <cmath>
#include <type_traits>

#if defined(__CUDACC__)
#define GLMS_FN __host__ __device__ __forceinline__
#else
#define GLMS_FN inline
#endif

namespace glm {

template <int N> struct vec;

template <> struct vec<2> {
    float x, y;
    GLMS_FN vec() : x(0.f), y(0.f) {}
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    GLMS_FN explicit vec(S s) : x(static_cast<float>(s)), y(static_cast<float>(s)) {}
    template <class A, class B>
    GLMS_FN vec(A a, B b) : x(static_cast<float>(a)), y(static_cast<float>(b)) {}
    GLMS_FN float& operator[](int i) { return (&x)[i]; }
    GLMS_FN const float& operator[](int i) const { return (&x)[i]; }
};

template <> struct vec<3> {
    float x, y, z;
    GLMS_FN vec() : x(0.f), y(0.f), z(0.f) {}
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    GLMS_FN explicit vec(S s) : x(static_cast<float>(s)), y(static_cast<float>(s)), z(static_cast<float>(s)) {}
    template <class A, class B, class C>
    GLMS_FN vec(A a, B b, C c) : x(static_cast<float>(a)), y(static_cast<float>(b)), z(static_cast<float>(c)) {}
    GLMS_FN explicit vec(const vec<4>& v);
    GLMS_FN float& operator[](int i) { return (&x)[i]; }
    GLMS_FN const float& operator[](int i) const { return (&x)[i]; }
};

template <> struct vec<4> {
    float x, y, z, w;
    GLMS_FN vec() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    GLMS_FN explicit vec(S s)
        : x(static_cast<float>(s)), y(static_cast<float>(s)), z(static_cast<float>(s)), w(static_cast<float>(s)) {}
    template <class A, class B, class C, class D>
    GLMS_FN vec(A a, B b, C c, D d)
        : x(static_cast<float>(a)), y(static_cast<float>(b)), z(static_cast<float>(c)), w(static_cast<float>(d)) {}
    template <class D>
    GLMS_FN vec(const vec<3>& v, D d) : x(v.x), y(v.y), z(v.z), w(static_cast<float>(d)) {}
    GLMS_FN float& operator[](int i) { return (&x)[i]; }
    GLMS_FN const float& operator[](int i) const { return (&x)[i]; }
};

GLMS_FN vec<3>::vec(const vec<4>& v) : x(v.x), y(v.y), z(v.z) {}

typedef vec<2> vec2;
typedef vec<3> vec3;
typedef vec<4> vec4;

static_assert(sizeof(vec2) == 8 && sizeof(vec3) == 12 && sizeof(vec4) == 16, "packed float vectors");

// ---- component-wise arithmetic --------------------------------------------

#define GLMS_VEC_BINOP(OP, OPEQ)                                                        \
    template <int N>                                                                    \
    GLMS_FN vec<N> operator OP(const vec<N>& a, const vec<N>& b) {                      \
        vec<N> r;                                                                       \
        for (int i = 0; i < N; ++i) r[i] = a[i] OP b[i];                                \
        return r;                                                                       \
    }                                                                                   \
    template <int N, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type> \
    GLMS_FN vec<N> operator OP(const vec<N>& a, S s) {                                  \
        const float f = static_cast<float>(s);                                          \
        vec<N> r;                                                                       \
        for (int i = 0; i < N; ++i) r[i] = a[i] OP f;                                   \
        return r;                                                                       \
    }                                                                                   \
    template <int N, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type> \
    GLMS_FN vec<N> operator OP(S s, const vec<N>& a) {                                  \
        const float f = static_cast<float>(s);                                          \
        vec<N> r;                                                                       \
        for (int i = 0; i < N; ++i) r[i] = f OP a[i];                                   \
        return r;                                                                       \
    }                                                                                   \
    template <int N>                                                                    \
    GLMS_FN vec<N>& operator OPEQ(vec<N>& a, const vec<N>& b) {                         \
        for (int i = 0; i < N; ++i) a[i] = a[i] OP b[i];                                \
        return a;                                                                       \
    }                                                                                   \
    template <int N, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type> \
    GLMS_FN vec<N>& operator OPEQ(vec<N>& a, S s) {                                     \
        const float f = static_cast<float>(s);                                          \
        for (int i = 0; i < N; ++i) a[i] = a[i] OP f;                                   \
        return a;                                                                       \
    }

GLMS_VEC_BINOP(+, +=)
GLMS_VEC_BINOP(-, -=)
GLMS_VEC_BINOP(*, *=)
GLMS_VEC_BINOP(/, /=)
#undef GLMS_VEC_BINOP

template <int N>
GLMS_FN vec<N> operator-(const vec<N>& a) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = -a[i];
    return r;
}

template <int N>
GLMS_FN vec<N> operator+(const vec<N>& a) { return a; }

// ---- geometric functions ----------------------------------------------------

template <int N>
GLMS_FN float dot(const vec<N>& a, const vec<N>& b) {
    float s = a[0] * b[0];
    for (int i = 1; i < N; ++i) s = s + a[i] * b[i];
    return s;
}

template <int N>
GLMS_FN float length(const vec<N>& a) { return sqrtf(dot(a, a)); }

template <int N>
GLMS_FN vec<N> normalize(const vec<N>& a) { return a * (1.0f / sqrtf(dot(a, a))); }

GLMS_FN vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

template <int N>
GLMS_FN vec<N> max(const vec<N>& a, const vec<N>& b) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = (a[i] < b[i]) ? b[i] : a[i];
    return r;
}
template <int N>
GLMS_FN vec<N> max(const vec<N>& a, float s) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = (a[i] < s) ? s : a[i];
    return r;
}
template <int N>
GLMS_FN vec<N> min(const vec<N>& a, const vec<N>& b) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = (b[i] < a[i]) ? b[i] : a[i];
    return r;
}
template <int N>
GLMS_FN vec<N> min(const vec<N>& a, float s) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = (s < a[i]) ? s : a[i];
    return r;
}
template <int N>
GLMS_FN vec<N> sqrt(const vec<N>& a) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = sqrtf(a[i]);
    return r;
}
template <int N>
GLMS_FN vec<N> abs(const vec<N>& a) {
    vec<N> r;
    for (int i = 0; i < N; ++i) r[i] = fabsf(a[i]);
    return r;
}

// ---- matrices: C columns of R rows ------------------------------------------

template <int C, int R> struct mat {
    vec<R> col[C];

    GLMS_FN mat() {
        for (int c = 0; c < C; ++c) col[c] = vec<R>(0.f);
    }
    // diagonal matrix
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    GLMS_FN explicit mat(S s) {
        for (int c = 0; c < C; ++c) {
            col[c] = vec<R>(0.f);
            if (c < R) col[c][c] = static_cast<float>(s);
        }
    }
    // C*R scalars, column after column
    template <class... A,
              class = typename std::enable_if<(sizeof...(A) == C * R) && (C * R > 1) &&
                                              std::conjunction<std::is_arithmetic<A>...>::value>::type>
    GLMS_FN mat(A... a) {
        const float v[C * R] = {static_cast<float>(a)...};
        for (int c = 0; c < C; ++c)
            for (int r = 0; r < R; ++r) col[c][r] = v[c * R + r];
    }
    // columns
    template <class... V,
              class = typename std::enable_if<(sizeof...(V) == C) &&
                                              std::conjunction<std::is_same<V, vec<R>>...>::value>::type,
              int = 0>
    GLMS_FN mat(const V&... v) {
        const vec<R> cols[C] = {v...};
        for (int c = 0; c < C; ++c) col[c] = cols[c];
    }

    GLMS_FN vec<R>& operator[](int c) { return col[c]; }
    GLMS_FN const vec<R>& operator[](int c) const { return col[c]; }
};

typedef mat<3, 3> mat3;
typedef mat<4, 4> mat4;
typedef mat<3, 4> mat3x4;   // 3 columns, 4 rows
typedef mat<4, 3> mat4x3;   // 4 columns, 3 rows
typedef mat<2, 2> mat2;

template <int C, int R>
GLMS_FN mat<R, C> transpose(const mat<C, R>& m) {
    mat<R, C> t;
    for (int c = 0; c < C; ++c)
        for (int r = 0; r < R; ++r) t[r][c] = m[c][r];
    return t;
}

// (A * B)[j][i] = sum_k A[k][i] * B[j][k]
template <int K, int R, int C>
GLMS_FN mat<C, R> operator*(const mat<K, R>& a, const mat<C, K>& b) {
    mat<C, R> out;
    for (int j = 0; j < C; ++j)
        for (int i = 0; i < R; ++i) {
            float s = a[0][i] * b[j][0];
            for (int k = 1; k < K; ++k) s = s + a[k][i] * b[j][k];
            out[j][i] = s;
        }
    return out;
}

// column vector: (m * v)[i] = sum_k m[k][i] * v[k]
template <int C, int R>
GLMS_FN vec<R> operator*(const mat<C, R>& m, const vec<C>& v) {
    vec<R> out;
    for (int i = 0; i < R; ++i) {
        float s = m[0][i] * v[0];
        for (int k = 1; k < C; ++k) s = s + m[k][i] * v[k];
        out[i] = s;
    }
    return out;
}

// row vector: (v * m)[j] = sum_k v[k] * m[j][k]
template <int C, int R>
GLMS_FN vec<C> operator*(const vec<R>& v, const mat<C, R>& m) {
    vec<C> out;
    for (int j = 0; j < C; ++j) {
        float s = m[j][0] * v[0];
        for (int k = 1; k < R; ++k) s = s + m[j][k] * v[k];
        out[j] = s;
    }
    return out;
}

template <int C, int R>
GLMS_FN mat<C, R> operator+(const mat<C, R>& a, const mat<C, R>& b) {
    mat<C, R> out;
    for (int c = 0; c < C; ++c) out[c] = a[c] + b[c];
    return out;
}

template <int C, int R>
GLMS_FN mat<C, R> operator-(const mat<C, R>& a, const mat<C, R>& b) {
    mat<C, R> out;
    for (int c = 0; c < C; ++c) out[c] = a[c] - b[c];
    return out;
}

template <int C, int R, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
GLMS_FN mat<C, R> operator*(const mat<C, R>& a, S s) {
    mat<C, R> out;
    for (int c = 0; c < C; ++c) out[c] = a[c] * s;
    return out;
}

template <int C, int R, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
GLMS_FN mat<C, R> operator*(S s, const mat<C, R>& a) {
    return a * s;
}

}  // namespace glm

#undef GLMS_FN
