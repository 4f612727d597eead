/*
 * tad/Scalar.cuh -- forward-mode second-order scalar for device code.
 *
 * Same semantics as TinyAD's Scalar<k, PassiveT, with_hessian>
 * (include/TinyAD/Scalar.hh:24-1347): a value, a dense k-gradient and a k x k
 * Hessian propagated through every operation by the chain rule; comparisons
 * look at the value only.  `Double<k>` / `Float<k>` are the aliases of
 * Scalar.hh:1389-1391.
 *
 * GB300 layout: the Hessian is symmetric, so only its upper triangle is
 * stored, packed row-major (k(k+1)/2 entries: 21 for k = 6, 78 for k = 12).
 * Every loop runs over compile-time k and unrolls, so a Scalar lives in
 * registers and each operation costs half the FMAs of the dense form.  The
 * optional `HR0, HC0` block restriction of the reference (a rectangular
 * Hessian block, used for mixed second derivatives, Scalar.hh:24, :186-196)
 * is provided by MixedScalar below.
 *
 * Precision split: Scalar<k, T, with_hessian, V, G> keeps the value in V,
 * the gradient in G and the Hessian in T.  Mixed<k> = Scalar<k, float, true,
 * double, DoubleFloat> is the mixed-precision scalar: values (edge vectors,
 * Jacobian determinants and inverses, the energy) are FP64, the O(k)
 * gradient is double-float (two FP32 words, ~1e-14 relative), and the
 * O(k^2) Hessian arithmetic is FP32.  A near-FP64 gradient keeps the Newton
 * fixed point, and the gradient's components along (near-)null directions of
 * the Hessian such as rigid motions, accurate; an FP32 gradient does not.
 * With V = G = T it is the reference's plain scalar.
 *
 * All functions are __host__ __device__ so element functors can be written
 * once and run on either side.
 */
#pragma once

#include <cmath>
#include <type_traits>

#if defined(__CUDACC__)
#define TAD_HD __host__ __device__ __forceinline__
#else
#define TAD_HD inline
#endif

namespace tad {

/* index of (i, j), i <= j, in the packed upper triangle of a k x k matrix */
TAD_HD constexpr int packed_index(int i, int j, int k) { return i * k - (i * (i - 1)) / 2 + (j - i); }

/* ---------------------------------------------------------------------------
 * DoubleFloat: an unevaluated sum hi + lo of two floats (~48-bit mantissa),
 * the gradient type of the mixed-precision scalar.  On GB300 a float FMA
 * issues at 70x the rate of a double one, so these few-FMA sequences carry
 * the gradient at near-FP64 accuracy (relative ~1e-14) for a fraction of an
 * FP64 instruction's cost.  Published algorithms: two-sum (Knuth, TAOCP vol.
 * 2, 4.2.2), the FMA two-product and Dekker's double-length arithmetic
 * (T. J. Dekker, "A floating-point technique for extending the available
 * precision", Numer. Math. 18, 1971).
 * ------------------------------------------------------------------------ */
struct DoubleFloat
{
    float hi, lo;
    TAD_HD DoubleFloat() : hi(0.f), lo(0.f) {}
    TAD_HD DoubleFloat(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    TAD_HD DoubleFloat(float h, float l) : hi(h), lo(l) {}
    TAD_HD explicit operator double() const { return float_to_double(hi) + float_to_double(lo); }
    TAD_HD explicit operator float() const { return hi + lo; }

    /* exact float -> double; on the device by bit construction for normal
       floats (the conversion instruction runs on the FP64 pipe) */
    TAD_HD static double float_to_double(float v)
    {
#if defined(__CUDA_ARCH__)
        const unsigned u = (unsigned)__float_as_int(v);
        const unsigned ex = (u >> 23) & 0xffu;
        if (ex != 0u && ex != 0xffu)
            return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                                    ((unsigned long long)(ex + 896u) << 52) |
                                                    ((unsigned long long)(u & 0x7fffffu) << 29)));
        if ((u << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)(u & 0x80000000u) << 32));
#endif
        return (double)v;
    }
};

TAD_HD DoubleFloat df_quick_two_sum(float a, float b)
{
    const float s = a + b;
    return DoubleFloat(s, b - (s - a));
}
TAD_HD DoubleFloat operator+(DoubleFloat a, DoubleFloat b)
{
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (b.hi - bb);     // two-sum error
    return df_quick_two_sum(s, e + a.lo + b.lo);
}
TAD_HD DoubleFloat operator-(DoubleFloat a) { return DoubleFloat(-a.hi, -a.lo); }
TAD_HD DoubleFloat operator-(DoubleFloat a, DoubleFloat b) { return a + (-b); }
TAD_HD DoubleFloat operator*(DoubleFloat a, DoubleFloat b)
{
    const float p = a.hi * b.hi;
#if defined(__CUDA_ARCH__)
    float e = __fmaf_rn(a.hi, b.hi, -p);                 // exact product error
#else
    float e = std::fma(a.hi, b.hi, -p);
#endif
    e += a.hi * b.lo + a.lo * b.hi;
    return df_quick_two_sum(p, e);
}
TAD_HD DoubleFloat& operator+=(DoubleFloat& a, DoubleFloat b) { a = a + b; return a; }

/* x y + z w with one renormalisation: both Dekker products through FMA,
   Knuth's two-sum of the high parts, the cross terms and rounding errors
   gathered in the low part (the product and quotient rules of the gradient) */
TAD_HD DoubleFloat df_dot2(DoubleFloat x, DoubleFloat y, DoubleFloat z, DoubleFloat w)
{
#if defined(__CUDA_ARCH__)
#define TAD_DF_FMA __fmaf_rn
#else
#define TAD_DF_FMA std::fma
#endif
    const float p1 = x.hi * y.hi, p2 = z.hi * w.hi;
    const float e1 = TAD_DF_FMA(x.hi, y.hi, -p1), e2 = TAD_DF_FMA(z.hi, w.hi, -p2);
    const float s = p1 + p2;
    const float v = s - p1;
    float lo = ((p1 - (s - v)) + (p2 - v)) + (e1 + e2);
    lo = TAD_DF_FMA(x.hi, y.lo, lo);
    lo = TAD_DF_FMA(x.lo, y.hi, lo);
    lo = TAD_DF_FMA(z.hi, w.lo, lo);
    lo = TAD_DF_FMA(z.lo, w.hi, lo);
#undef TAD_DF_FMA
    return df_quick_two_sum(s, lo);
}
/* x y + z w in the gradient type (fused for the double-float gradient) */
template <typename G> TAD_HD G grad_dot2(const G& x, const G& y, const G& z, const G& w) { return x * y + z * w; }
template <> TAD_HD DoubleFloat grad_dot2<DoubleFloat>(const DoubleFloat& x, const DoubleFloat& y, const DoubleFloat& z,
                                                      const DoubleFloat& w)
{
    return df_dot2(x, y, z, w);
}
TAD_HD bool isfinite(DoubleFloat a) { using std::isfinite; return isfinite(a.hi) && isfinite(a.lo); }

/* Value channel of the mixed-precision scalar: the unevaluated sum hi + lo of
   two floats (a ~48-bit significand) computed on the FP32 pipe, so that no
   FP64 instruction or double <-> float conversion is left inside the
   per-operation work of a mixed element kernel.  Unlike the gradient's
   DoubleFloat it carries the full passive semantics element functors rely
   on: accurate addition (two-sum on both parts, so differences such as
   determinants keep their relative accuracy), division and square root (the
   float quotient / root plus one Newton correction computed from the exact
   FMA residual), comparisons, the elementary functions (evaluated in double
   and split back; rare in energies), and IEEE propagation of infinities and
   NaNs (a non-finite hi part travels with lo = 0).  Methods: Knuth's
   two-sum, Dekker's product (here via FMA) and the double-double division
   and square root of Hida, Li and Bailey (2001), in float. */
struct DoubleFloatValue
{
    float hi, lo;
    TAD_HD DoubleFloatValue() : hi(0.f), lo(0.f) {}
    TAD_HD DoubleFloatValue(double x) : hi(0.f), lo(0.f)
    {
#if defined(__CUDA_ARCH__)
        // Bit-level split with integer and FP32 instructions only (every
        // branch: a short FP64 fallback would be if-converted and issued for
        // all threads).  hi = the sign, exponent and top 23 stored mantissa
        // bits of x (x truncated to float precision, exact); lo = the
        // remaining 29 mantissa bits rounded to nearest float and scaled by
        // the exact power of two 2^(e - 1075) (|lo| < ulp(hi); the split is
        // within 2^-49 |x|).  The 29-bit integer becomes a float without a
        // conversion instruction: for v < 2^23 the float with bits
        // 0x4b000000 | v is exactly 2^23 + v, so both halves convert exactly
        // by one subtraction and one FMA rounds rh 2^23 + rl once.  Below the
        // normal float range x becomes a signed zero, above it +-inf; NaN
        // stays NaN.
        const unsigned long long b = (unsigned long long)__double_as_longlong(x);
        const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
        const int e = (int)((b >> 52) & 0x7ff);
        if (e >= 897 && e <= 1150)
        {
            hi = __int_as_float((int)(sign | ((unsigned)(e - 896) << 23) | ((unsigned)(b >> 29) & 0x7fffffu)));
            const unsigned r = (unsigned)b & 0x1fffffffu;
            const float rh = __int_as_float((int)(0x4b000000u | (r >> 23))) - 8388608.0f;
            const float rl = __int_as_float((int)(0x4b000000u | (r & 0x7fffffu))) - 8388608.0f;
            const float rf = __fmaf_rn(rh, 8388608.0f, rl);
            if (e >= 949) lo = rf * __int_as_float((int)((unsigned)(e - 948) << 23));              // 2^(e - 1075)
            else lo = (rf * __int_as_float((int)((unsigned)(e - 884) << 23))) * 5.42101086242752217e-20f;  // 2^(e - 1011) 2^-64
            if (sign) lo = -lo;
        }
        else if (e == 2047)
            hi = __int_as_float((int)(sign | 0x7f800000u | ((b & 0xfffffffffffffull) ? 0x400000u : 0u)));
        else if (e > 1150)
            hi = __int_as_float((int)(sign | 0x7f800000u));
        else
            hi = __int_as_float((int)sign);
#else
        hi = (float)x;
        using std::isfinite;
        if (isfinite(hi)) lo = (float)(x - (double)hi);
#endif
    }
    TAD_HD DoubleFloatValue(float x) : hi(x), lo(0.f) {}
    template <typename I, typename = std::enable_if_t<std::is_integral<I>::value>>
    TAD_HD DoubleFloatValue(I x) : DoubleFloatValue((double)x) {}
    TAD_HD DoubleFloatValue(float h, float l) : hi(h), lo(l) {}
    TAD_HD explicit operator double() const { return DoubleFloat::float_to_double(hi) + DoubleFloat::float_to_double(lo); }
    TAD_HD explicit operator float() const { return hi + lo; }
    TAD_HD explicit operator DoubleFloat() const { return DoubleFloat(hi, lo); }
};

TAD_HD float dfv_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
TAD_HD bool dfv_finite(float v) { using std::isfinite; return isfinite(v); }
TAD_HD DoubleFloatValue dfv_quick(float s, float e)
{
    const float t = s + e;
    return DoubleFloatValue(t, e - (t - s));
}
TAD_HD DoubleFloatValue operator+(DoubleFloatValue a, DoubleFloatValue b)
{
    const float s = a.hi + b.hi;
    if (!dfv_finite(s)) return DoubleFloatValue(s, 0.f);
    const float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);
    const float t = a.lo + b.lo;
    const float w = t - a.lo;
    const float f = (a.lo - (t - w)) + (b.lo - w);
    // full two-sum here: when the hi parts cancel, e + t can exceed s
    e += t;
    const float r = s + e;
    const float z = r - s;
    const float rl = (s - (r - z)) + (e - z);
    return dfv_quick(r, rl + f);
}
TAD_HD DoubleFloatValue operator-(DoubleFloatValue a) { return DoubleFloatValue(-a.hi, -a.lo); }
TAD_HD DoubleFloatValue operator-(DoubleFloatValue a, DoubleFloatValue b) { return a + (-b); }
TAD_HD DoubleFloatValue operator*(DoubleFloatValue a, DoubleFloatValue b)
{
    const float p = a.hi * b.hi;
    if (!dfv_finite(p)) return DoubleFloatValue(p, 0.f);
    float e = dfv_fma(a.hi, b.hi, -p);
    e = dfv_fma(a.hi, b.lo, e);
    e = dfv_fma(a.lo, b.hi, e);
    return dfv_quick(p, e);
}
TAD_HD DoubleFloatValue operator/(DoubleFloatValue a, DoubleFloatValue b)
{
    const float q1 = a.hi / b.hi;
    if (!dfv_finite(q1) || !dfv_finite(b.hi) || q1 == 0.f) return DoubleFloatValue(q1, 0.f);
    // a - q1 b, with q1 b.hi exact through the FMA residual
    const float ph = q1 * b.hi;
    const float pl = dfv_fma(q1, b.lo, dfv_fma(q1, b.hi, -ph));
    const float r = ((a.hi - ph) - pl) + a.lo;
    return dfv_quick(q1, r / b.hi);
}
TAD_HD DoubleFloatValue& operator+=(DoubleFloatValue& a, DoubleFloatValue b) { a = a + b; return a; }
TAD_HD DoubleFloatValue& operator-=(DoubleFloatValue& a, DoubleFloatValue b) { a = a - b; return a; }
TAD_HD DoubleFloatValue& operator*=(DoubleFloatValue& a, DoubleFloatValue b) { a = a * b; return a; }
TAD_HD DoubleFloatValue& operator/=(DoubleFloatValue& a, DoubleFloatValue b) { a = a / b; return a; }
TAD_HD bool operator<(DoubleFloatValue a, DoubleFloatValue b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
TAD_HD bool operator>(DoubleFloatValue a, DoubleFloatValue b) { return b < a; }
TAD_HD bool operator<=(DoubleFloatValue a, DoubleFloatValue b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
TAD_HD bool operator>=(DoubleFloatValue a, DoubleFloatValue b) { return b <= a; }
TAD_HD bool operator==(DoubleFloatValue a, DoubleFloatValue b) { return a.hi == b.hi && a.lo == b.lo; }
TAD_HD bool operator!=(DoubleFloatValue a, DoubleFloatValue b) { return !(a == b); }
TAD_HD DoubleFloatValue sqrt(DoubleFloatValue a)
{
    using std::sqrt;
    const float y = sqrt(a.hi);
    if (!(a.hi > 0.f) || !dfv_finite(a.hi)) return DoubleFloatValue(y, 0.f);
    // a - y^2 from the exact square (FMA residual), then y + (a - y^2) / (2y)
    const float yy = y * y;
    const float r = ((a.hi - yy) - dfv_fma(y, y, -yy)) + a.lo;
    return dfv_quick(y, r / (2.f * y));
}
TAD_HD DoubleFloatValue fabs(DoubleFloatValue a) { return a.hi < 0.f ? -a : a; }
TAD_HD DoubleFloatValue abs(DoubleFloatValue a) { return fabs(a); }
TAD_HD DoubleFloatValue sqr(DoubleFloatValue a) { return a * a; }
TAD_HD bool isfinite(DoubleFloatValue a) { return dfv_finite(a.hi); }
TAD_HD bool isnan(DoubleFloatValue a) { using std::isnan; return isnan(a.hi); }
TAD_HD bool isinf(DoubleFloatValue a) { using std::isinf; return isinf(a.hi); }
#define TAD_DFV_VIA_DOUBLE(F)                                                                              \
    TAD_HD DoubleFloatValue F(DoubleFloatValue a) { using std::F; return DoubleFloatValue(F((double)a)); }
TAD_DFV_VIA_DOUBLE(exp)
TAD_DFV_VIA_DOUBLE(log)
TAD_DFV_VIA_DOUBLE(log2)
TAD_DFV_VIA_DOUBLE(log10)
TAD_DFV_VIA_DOUBLE(sin)
TAD_DFV_VIA_DOUBLE(cos)
TAD_DFV_VIA_DOUBLE(tan)
TAD_DFV_VIA_DOUBLE(asin)
TAD_DFV_VIA_DOUBLE(acos)
TAD_DFV_VIA_DOUBLE(atan)
TAD_DFV_VIA_DOUBLE(sinh)
TAD_DFV_VIA_DOUBLE(cosh)
TAD_DFV_VIA_DOUBLE(tanh)
TAD_DFV_VIA_DOUBLE(asinh)
TAD_DFV_VIA_DOUBLE(acosh)
TAD_DFV_VIA_DOUBLE(atanh)
#undef TAD_DFV_VIA_DOUBLE
TAD_HD DoubleFloatValue atan2(DoubleFloatValue y, DoubleFloatValue x) { using std::atan2; return DoubleFloatValue(atan2((double)y, (double)x)); }
TAD_HD DoubleFloatValue pow(DoubleFloatValue a, DoubleFloatValue e) { using std::pow; return DoubleFloatValue(pow((double)a, (double)e)); }
TAD_HD DoubleFloatValue pow(DoubleFloatValue a, int e) { using std::pow; return DoubleFloatValue(pow((double)a, e)); }

template <int K, typename T, bool WithHessian = true, typename V = T, typename G = V>
struct Scalar
{
    static constexpr int k = K;
    static constexpr bool with_hessian = WithHessian;
    static constexpr int n_hess = WithHessian ? K * (K + 1) / 2 : 0;
    using passive_type = V;
    using grad_type = G;
    using deriv_type = T;

    V val;
    G grad[K];
    T hess[n_hess > 0 ? n_hess : 1];

    TAD_HD Scalar() : val(V(0))
    {
#pragma unroll
        for (int i = 0; i < K; ++i) grad[i] = G(0);
#pragma unroll
        for (int i = 0; i < (n_hess > 0 ? n_hess : 1); ++i) hess[i] = T(0);
    }

    /* passive constant (Scalar.hh:58-63) */
    TAD_HD Scalar(V v) : Scalar() { val = v; }
    template <typename U, typename = std::enable_if_t<std::is_arithmetic<U>::value && !std::is_same<U, V>::value>>
    TAD_HD Scalar(U v) : Scalar() { val = V(v); }

    /* active variable with index idx (Scalar.hh:67-75) */
    TAD_HD Scalar(V v, int idx) : Scalar()
    {
        val = v;
#pragma unroll
        for (int i = 0; i < K; ++i) grad[i] = (i == idx) ? G(1) : G(0);
    }

    /* univariate known derivatives (Scalar.hh:89-101) */
    TAD_HD static Scalar known_derivatives(V v, G g, T h)
    {
        Scalar r(v);
        r.grad[0] = g;
        if (WithHessian) r.hess[0] = h;
        return r;
    }

    /* full-matrix read access to the Hessian */
    TAD_HD T H(int i, int j) const { return i <= j ? hess[packed_index(i, j, K)] : hess[packed_index(j, i, K)]; }

    /* the gradient in the Hessian's precision */
    TAD_HD void grad_as_hess_type(T (&t)[K]) const
    {
#pragma unroll
        for (int i = 0; i < K; ++i) t[i] = T(grad[i]);
    }

    /* chain rule for f(a) with f, f', f'' known (Scalar.hh:199-214):
       grad = f' ga, Hess = f'' ga ga^T + f' Ha */
    TAD_HD static Scalar chain(V f, V f1v, V f2v, const Scalar& a)
    {
        Scalar r;
        r.val = f;
        const G f1g = G(f1v);
#pragma unroll
        for (int i = 0; i < K; ++i) r.grad[i] = f1g * a.grad[i];
        if (WithHessian)
        {
            const T f1 = T(f1v), f2 = T(f2v);
            T ta[K];
            a.grad_as_hess_type(ta);
            int q = 0;
#pragma unroll
            for (int i = 0; i < K; ++i)
            {
                const T fgi = f2 * ta[i];
#pragma unroll
                for (int j = i; j < K; ++j, ++q) r.hess[q] = fgi * ta[j] + f1 * a.hess[q];
            }
        }
        return r;
    }
};

template <int K, bool WithHessian = true> using Double = Scalar<K, double, WithHessian>;
template <int K, bool WithHessian = true> using Float = Scalar<K, float, WithHessian>;
/* mixed precision: double-float value and gradient, FP32 Hessian */
template <int K, bool WithHessian = true> using Mixed = Scalar<K, float, WithHessian, DoubleFloatValue, DoubleFloat>;

template <typename S> struct is_scalar : std::false_type {};
template <int K, typename T, bool H, typename V, typename G> struct is_scalar<Scalar<K, T, H, V, G>> : std::true_type {};

/* ---- passive helpers: to_passive / value_of ---------------------------- */
template <typename T, typename = std::enable_if_t<std::is_arithmetic<T>::value>>
TAD_HD T to_passive(T v) { return v; }
template <int K, typename T, bool H, typename V, typename G>
TAD_HD V to_passive(const Scalar<K, T, H, V, G>& a) { return a.val; }

#define TAD_S Scalar<K, T, H, V, G>
#define TAD_TPL template <int K, typename T, bool H, typename V, typename G>
#define TAD_TPLU template <int K, typename T, bool H, typename V, typename G, typename U, typename = std::enable_if_t<std::is_arithmetic<U>::value || std::is_same<U, V>::value>>

/* ---- unary -------------------------------------------------------------- */
TAD_TPL TAD_HD TAD_S operator-(const TAD_S& a)                              // Scalar.hh:220-234
{
    TAD_S r;
    r.val = -a.val;
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = -a.grad[i];
#pragma unroll
    for (int i = 0; i < TAD_S::n_hess; ++i) r.hess[i] = -a.hess[i];
    return r;
}
TAD_TPL TAD_HD TAD_S operator+(const TAD_S& a) { return a; }

TAD_TPL TAD_HD TAD_S sqrt(const TAD_S& a)                                    // Scalar.hh:236-247
{
    using std::sqrt;
    const V f = sqrt(a.val);
    return TAD_S::chain(f, V(0.5) / f, V(-0.25) / (f * a.val), a);
}

TAD_TPL TAD_HD TAD_S sqr(const TAD_S& a)                                     // Scalar.hh:249-264
{
    TAD_S r;
    r.val = a.val * a.val;
    const G two_vg = G(V(2) * a.val);
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = two_vg * a.grad[i];
    if (H)
    {
        const T two_v = T(V(2) * a.val);
        T ta[K];
        a.grad_as_hess_type(ta);
        int q = 0;
#pragma unroll
        for (int i = 0; i < K; ++i)
        {
            const T gi2 = T(2) * ta[i];
#pragma unroll
            for (int j = i; j < K; ++j, ++q) r.hess[q] = two_v * a.hess[q] + gi2 * ta[j];
        }
    }
    return r;
}

TAD_TPL TAD_HD TAD_S pow(const TAD_S& a, int e)                              // Scalar.hh:266-289
{
    using std::pow;
    if (e == 0) return TAD_S::chain(V(1), V(0), V(0), a);
    if (e == 1) return TAD_S::chain(a.val, V(1), V(0), a);
    const V f2 = (V)pow(a.val, e - 2);
    const V f1 = f2 * a.val;
    return TAD_S::chain(f1 * a.val, V(e) * f1, V(e * (e - 1)) * f2, a);
}

template <int K, typename T, bool H, typename V, typename G, typename U, typename = std::enable_if_t<std::is_floating_point<U>::value || std::is_same<U, V>::value>>
TAD_HD TAD_S pow(const TAD_S& a, U eu)                                       // Scalar.hh:291-307
{
    using std::pow;
    const V e = V(eu);
    const V f2 = pow(a.val, e - V(2));
    const V f1 = f2 * a.val;
    return TAD_S::chain(f1 * a.val, e * f1, e * (e - V(1)) * f2, a);
}

TAD_TPL TAD_HD TAD_S exp(const TAD_S& a) { using std::exp; const V e = exp(a.val); return TAD_S::chain(e, e, e, a); }   // Scalar.hh:324-332
TAD_TPL TAD_HD TAD_S log(const TAD_S& a)                                                                               // Scalar.hh:334-346
{
    using std::log;
    const V ai = V(1) / a.val;
    return TAD_S::chain(log(a.val), ai, -ai * ai, a);
}
TAD_TPL TAD_HD TAD_S log2(const TAD_S& a)                                   // Scalar.hh:348-358
{
    using std::log; using std::log2;
    const V ai = V(1) / (a.val * V(log(2.0)));
    return TAD_S::chain(log2(a.val), ai, -ai / a.val, a);
}
TAD_TPL TAD_HD TAD_S log10(const TAD_S& a)                                  // Scalar.hh:360-370
{
    using std::log; using std::log10;
    const V ai = V(1) / (a.val * V(log(10.0)));
    return TAD_S::chain(log10(a.val), ai, -ai / a.val, a);
}
TAD_TPL TAD_HD TAD_S sin(const TAD_S& a) { using std::sin; using std::cos; const V s = sin(a.val); return TAD_S::chain(s, cos(a.val), -s, a); }
TAD_TPL TAD_HD TAD_S cos(const TAD_S& a) { using std::sin; using std::cos; const V c = cos(a.val); return TAD_S::chain(c, -sin(a.val), -c, a); }
TAD_TPL TAD_HD TAD_S tan(const TAD_S& a)
{
    using std::tan; using std::cos; using std::sin;
    const V c = cos(a.val);
    const V c2 = c * c;
    return TAD_S::chain(tan(a.val), V(1) / c2, V(2) * sin(a.val) / (c2 * c), a);
}
TAD_TPL TAD_HD TAD_S asin(const TAD_S& a)
{
    using std::asin; using std::sqrt;
    const V s = V(1) - a.val * a.val;
    const V ss = sqrt(s);
    return TAD_S::chain(asin(a.val), V(1) / ss, a.val / (ss * s), a);
}
TAD_TPL TAD_HD TAD_S acos(const TAD_S& a)
{
    using std::acos; using std::sqrt;
    const V s = V(1) - a.val * a.val;
    const V ss = sqrt(s);
    return TAD_S::chain(acos(a.val), V(-1) / ss, -a.val / (ss * s), a);
}
TAD_TPL TAD_HD TAD_S atan(const TAD_S& a)
{
    using std::atan;
    const V s = a.val * a.val + V(1);
    return TAD_S::chain(atan(a.val), V(1) / s, V(-2) * a.val / (s * s), a);
}
TAD_TPL TAD_HD TAD_S sinh(const TAD_S& a) { using std::sinh; using std::cosh; const V s = sinh(a.val); return TAD_S::chain(s, cosh(a.val), s, a); }
TAD_TPL TAD_HD TAD_S cosh(const TAD_S& a) { using std::sinh; using std::cosh; const V c = cosh(a.val); return TAD_S::chain(c, sinh(a.val), c, a); }
TAD_TPL TAD_HD TAD_S tanh(const TAD_S& a)
{
    using std::tanh; using std::cosh; using std::sinh;
    const V c = cosh(a.val);
    const V c2 = c * c;
    return TAD_S::chain(tanh(a.val), V(1) / c2, V(-2) * sinh(a.val) / (c2 * c), a);
}
TAD_TPL TAD_HD TAD_S asinh(const TAD_S& a)                                  // Scalar.hh:501-515
{
    using std::asinh; using std::sqrt;
    const V s = a.val * a.val + V(1);
    const V ss = sqrt(s);
    return TAD_S::chain(asinh(a.val), V(1) / ss, -a.val / (ss * s), a);
}
TAD_TPL TAD_HD TAD_S acosh(const TAD_S& a)                                  // Scalar.hh:517-534
{
    using std::acosh; using std::sqrt;
    const V sm = a.val - V(1), sp = a.val + V(1);
    const V prod = sqrt(sm) * sqrt(sp);
    return TAD_S::chain(acosh(a.val), V(1) / prod, -a.val / (prod * sm * sp), a);
}
TAD_TPL TAD_HD TAD_S atanh(const TAD_S& a)                                  // Scalar.hh:536-546
{
    using std::atanh;
    const V s = V(1) - a.val * a.val;
    return TAD_S::chain(atanh(a.val), V(1) / s, V(2) * a.val / (s * s), a);
}
TAD_TPL TAD_HD TAD_S fabs(const TAD_S& a)                                   // Scalar.hh:309-322
{
    return a.val >= V(0) ? TAD_S::chain(a.val, V(1), V(0), a) : TAD_S::chain(-a.val, V(-1), V(0), a);
}
TAD_TPL TAD_HD TAD_S abs(const TAD_S& a) { return fabs(a); }

TAD_TPL TAD_HD bool isnan(const TAD_S& a) { using std::isnan; return isnan(a.val); }
TAD_TPL TAD_HD bool isinf(const TAD_S& a) { using std::isinf; return isinf(a.val); }
TAD_TPL TAD_HD bool isfinite(const TAD_S& a) { using std::isfinite; return isfinite(a.val); }

/* ---- binary: + - -------------------------------------------------------- */
TAD_TPL TAD_HD TAD_S operator+(const TAD_S& a, const TAD_S& b)              // Scalar.hh:579-595
{
    TAD_S r;
    r.val = a.val + b.val;
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = a.grad[i] + b.grad[i];
#pragma unroll
    for (int i = 0; i < TAD_S::n_hess; ++i) r.hess[i] = a.hess[i] + b.hess[i];
    return r;
}
TAD_TPL TAD_HD TAD_S operator-(const TAD_S& a, const TAD_S& b)              // Scalar.hh:651-667
{
    TAD_S r;
    r.val = a.val - b.val;
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = a.grad[i] - b.grad[i];
#pragma unroll
    for (int i = 0; i < TAD_S::n_hess; ++i) r.hess[i] = a.hess[i] - b.hess[i];
    return r;
}
TAD_TPLU TAD_HD TAD_S operator+(const TAD_S& a, U b) { TAD_S r = a; r.val += V(b); return r; }   // Scalar.hh:597-621
TAD_TPLU TAD_HD TAD_S operator+(U a, const TAD_S& b) { TAD_S r = b; r.val += V(a); return r; }
TAD_TPLU TAD_HD TAD_S operator-(const TAD_S& a, U b) { TAD_S r = a; r.val -= V(b); return r; }   // Scalar.hh:669-698
TAD_TPLU TAD_HD TAD_S operator-(U a, const TAD_S& b) { TAD_S r = -b; r.val += V(a); return r; }

/* ---- binary: * ---------------------------------------------------------- */
/* Hess(ab) = b Ha + ga gb^T + gb ga^T + a Hb (Scalar.hh:738-769) */
TAD_TPL TAD_HD TAD_S operator*(const TAD_S& a, const TAD_S& b)
{
    TAD_S r;
    r.val = a.val * b.val;
    const G avg = G(a.val), bvg = G(b.val);
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = grad_dot2(bvg, a.grad[i], avg, b.grad[i]);
    if (H)
    {
        const T av = T(a.val), bv = T(b.val);
        T ta[K], tb[K];
        a.grad_as_hess_type(ta);
        b.grad_as_hess_type(tb);
        int q = 0;
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = i; j < K; ++j, ++q)
                r.hess[q] = bv * a.hess[q] + ta[i] * tb[j] + tb[i] * ta[j] + av * b.hess[q];
    }
    return r;
}
TAD_TPLU TAD_HD TAD_S operator*(const TAD_S& a, U b)                        // Scalar.hh:771-786
{
    TAD_S r;
    r.val = a.val * V(b);
    const G sg = G(b);
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = a.grad[i] * sg;
    const T s = T(b);
#pragma unroll
    for (int i = 0; i < TAD_S::n_hess; ++i) r.hess[i] = a.hess[i] * s;
    return r;
}
TAD_TPLU TAD_HD TAD_S operator*(U a, const TAD_S& b) { return b * a; }

/* ---- binary: / ---------------------------------------------------------- */
/* r = a/b: grad = (ga - r gb)/b, Hess = (Ha - gr gb^T - gb gr^T - r Hb)/b
   (Scalar.hh:823-840; the reciprocal of b is taken once) */
TAD_TPL TAD_HD TAD_S operator/(const TAD_S& a, const TAD_S& b)
{
    TAD_S r;
    const V ibv = V(1) / b.val;
    r.val = a.val * ibv;
    const G ibg = G(ibv), rvg = G(r.val);
    if constexpr (std::is_same<G, DoubleFloat>::value)
    {
        // (ga - r gb) / b as one fused x y + z w per entry
        const G nrib = -(rvg * ibg);
#pragma unroll
        for (int i = 0; i < K; ++i) r.grad[i] = df_dot2(ibg, a.grad[i], nrib, b.grad[i]);
    }
    else
    {
#pragma unroll
        for (int i = 0; i < K; ++i) r.grad[i] = (a.grad[i] - rvg * b.grad[i]) * ibg;
    }
    if (H)
    {
        const T ib = T(ibv), rv = T(r.val);
        T tr[K], tb[K];
        r.grad_as_hess_type(tr);
        b.grad_as_hess_type(tb);
        int q = 0;
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = i; j < K; ++j, ++q)
                r.hess[q] = (a.hess[q] - tr[i] * tb[j] - tb[i] * tr[j] - rv * b.hess[q]) * ib;
    }
    return r;
}
TAD_TPLU TAD_HD TAD_S operator/(const TAD_S& a, U b)                        // Scalar.hh:842-857
{
    TAD_S r;
    const V ibv = V(1) / V(b);
    r.val = a.val * ibv;
    const G ibg = G(ibv);
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = a.grad[i] * ibg;
    const T ib = T(ibv);
#pragma unroll
    for (int i = 0; i < TAD_S::n_hess; ++i) r.hess[i] = a.hess[i] * ib;
    return r;
}
/* passive / Scalar (Scalar.hh:859-877): r = c/b, gr = -r gb / b,
   Hess = (-gr gb^T - gb gr^T - r Hb) / b */
TAD_TPLU TAD_HD TAD_S operator/(U c, const TAD_S& b)
{
    TAD_S r;
    const V ibv = V(1) / b.val;
    r.val = V(c) * ibv;
    const G sg = G(-r.val * ibv);
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = sg * b.grad[i];
    if (H)
    {
        const T ib = T(ibv), rv = T(r.val);
        T tr[K], tb[K];
        r.grad_as_hess_type(tr);
        b.grad_as_hess_type(tb);
        int q = 0;
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = i; j < K; ++j, ++q)
                r.hess[q] = -(tr[i] * tb[j] + tb[i] * tr[j] + rv * b.hess[q]) * ib;
    }
    return r;
}

TAD_TPL TAD_HD TAD_S& operator+=(TAD_S& a, const TAD_S& b) { a = a + b; return a; }
TAD_TPL TAD_HD TAD_S& operator-=(TAD_S& a, const TAD_S& b) { a = a - b; return a; }
TAD_TPL TAD_HD TAD_S& operator*=(TAD_S& a, const TAD_S& b) { a = a * b; return a; }
TAD_TPL TAD_HD TAD_S& operator/=(TAD_S& a, const TAD_S& b) { a = a / b; return a; }
TAD_TPLU TAD_HD TAD_S& operator+=(TAD_S& a, U b) { a.val += V(b); return a; }
TAD_TPLU TAD_HD TAD_S& operator-=(TAD_S& a, U b) { a.val -= V(b); return a; }
TAD_TPLU TAD_HD TAD_S& operator*=(TAD_S& a, U b) { a = a * b; return a; }
TAD_TPLU TAD_HD TAD_S& operator/=(TAD_S& a, U b) { a = a / b; return a; }

/* atan2 (Scalar.hh:891-915).  The full Hessian is symmetric; only i <= j is
   formed. */
TAD_TPL TAD_HD TAD_S atan2(const TAD_S& y, const TAD_S& x)
{
    using std::atan2;
    TAD_S r;
    r.val = atan2(y.val, x.val);
    const V ivv = V(1) / (x.val * x.val + y.val * y.val);
    const G ivg = G(ivv), xg = G(x.val), yg = G(y.val);
#pragma unroll
    for (int i = 0; i < K; ++i) r.grad[i] = (xg * y.grad[i] - yg * x.grad[i]) * ivg;
    if (H)
    {
        const T iv = T(ivv), xv = T(x.val), yv = T(y.val);
        T tx[K], ty[K], tr[K], dv[K];
        x.grad_as_hess_type(tx);
        y.grad_as_hess_type(ty);
        r.grad_as_hess_type(tr);
#pragma unroll
        for (int i = 0; i < K; ++i) dv[i] = T(2) * (xv * tx[i] + yv * ty[i]);
        int q = 0;
#pragma unroll
        for (int i = 0; i < K; ++i)
#pragma unroll
            for (int j = i; j < K; ++j, ++q)
            {
                const T du = xv * y.hess[q] - yv * x.hess[q] + ty[i] * tx[j] - tx[i] * ty[j];
                r.hess[q] = (du - tr[i] * dv[j]) * iv;
            }
    }
    return r;
}
TAD_TPL TAD_HD TAD_S hypot(const TAD_S& a, const TAD_S& b) { return sqrt(a * a + b * b); }   // Scalar.hh:917-926

/* ---- comparisons on the value (Scalar.hh:933-1095) ---------------------- */
#define TAD_CMP(OP)                                                                           \
    TAD_TPL TAD_HD bool operator OP(const TAD_S& a, const TAD_S& b) { return a.val OP b.val; } \
    TAD_TPLU TAD_HD bool operator OP(const TAD_S& a, U b) { return a.val OP V(b); }            \
    TAD_TPLU TAD_HD bool operator OP(U a, const TAD_S& b) { return V(a) OP b.val; }
TAD_CMP(==)
TAD_CMP(!=)
TAD_CMP(<)
TAD_CMP(<=)
TAD_CMP(>)
TAD_CMP(>=)
#undef TAD_CMP

TAD_TPL TAD_HD TAD_S min(const TAD_S& a, const TAD_S& b) { return (b < a) ? b : a; }
TAD_TPL TAD_HD TAD_S max(const TAD_S& a, const TAD_S& b) { return (a < b) ? b : a; }
TAD_TPL TAD_HD TAD_S fmin(const TAD_S& a, const TAD_S& b) { return min(a, b); }
TAD_TPL TAD_HD TAD_S fmax(const TAD_S& a, const TAD_S& b) { return max(a, b); }
TAD_TPL TAD_HD TAD_S clamp(const TAD_S& x, const TAD_S& a, const TAD_S& b) { return (x < a) ? a : ((x > b) ? b : x); }

#undef TAD_TPLU
#undef TAD_TPL
#undef TAD_S

/* passive overloads so functors written for Scalar also compile passively */
TAD_HD double sqr(double v) { return v * v; }
TAD_HD float sqr(float v) { return v * v; }

/* ---------------------------------------------------------------------------
 * MixedScalar<KX, KP, T>: value, full gradient over KX + KP variables and
 * only the KX x KP block d2f/dx dp of the Hessian -- the truncated-block
 * scalar Scalar<KX+KP, T, true, 0, KX, KX, KP> of the reference
 * (Scalar.hh:24, :186-196; pinned by tests/ScalarTestHessianBlock.cc).
 * The block is not symmetric and is stored dense, row-major.
 * ------------------------------------------------------------------------ */
template <int KX, int KP, typename T>
struct MixedScalar
{
    static constexpr int k = KX + KP;
    using passive_type = T;
    T val;
    T grad[KX + KP];
    T blk[KX * KP];

    TAD_HD MixedScalar() : val(T(0))
    {
#pragma unroll
        for (int i = 0; i < k; ++i) grad[i] = T(0);
#pragma unroll
        for (int i = 0; i < KX * KP; ++i) blk[i] = T(0);
    }
    TAD_HD MixedScalar(T v) : MixedScalar() { val = v; }
    TAD_HD MixedScalar(T v, int idx) : MixedScalar()
    {
        val = v;
#pragma unroll
        for (int i = 0; i < k; ++i) grad[i] = (i == idx) ? T(1) : T(0);
    }
    TAD_HD static MixedScalar chain(T f, T f1, T f2, const MixedScalar& a)
    {
        MixedScalar r;
        r.val = f;
#pragma unroll
        for (int i = 0; i < k; ++i) r.grad[i] = f1 * a.grad[i];
#pragma unroll
        for (int i = 0; i < KX; ++i)
#pragma unroll
            for (int j = 0; j < KP; ++j)
                r.blk[i * KP + j] = f2 * a.grad[i] * a.grad[KX + j] + f1 * a.blk[i * KP + j];
        return r;
    }
};

#define TAD_M MixedScalar<KX, KP, T>
#define TAD_TPL template <int KX, int KP, typename T>
#define TAD_TPLU template <int KX, int KP, typename T, typename U, typename = std::enable_if_t<std::is_arithmetic<U>::value>>
TAD_TPL TAD_HD TAD_M operator-(const TAD_M& a)
{
    TAD_M r; r.val = -a.val;
#pragma unroll
    for (int i = 0; i < KX + KP; ++i) r.grad[i] = -a.grad[i];
#pragma unroll
    for (int i = 0; i < KX * KP; ++i) r.blk[i] = -a.blk[i];
    return r;
}
TAD_TPL TAD_HD TAD_M operator+(const TAD_M& a, const TAD_M& b)
{
    TAD_M r; r.val = a.val + b.val;
#pragma unroll
    for (int i = 0; i < KX + KP; ++i) r.grad[i] = a.grad[i] + b.grad[i];
#pragma unroll
    for (int i = 0; i < KX * KP; ++i) r.blk[i] = a.blk[i] + b.blk[i];
    return r;
}
TAD_TPL TAD_HD TAD_M operator-(const TAD_M& a, const TAD_M& b) { return a + (-b); }
TAD_TPL TAD_HD TAD_M operator*(const TAD_M& a, const TAD_M& b)
{
    TAD_M r; r.val = a.val * b.val;
#pragma unroll
    for (int i = 0; i < KX + KP; ++i) r.grad[i] = b.val * a.grad[i] + a.val * b.grad[i];
#pragma unroll
    for (int i = 0; i < KX; ++i)
#pragma unroll
        for (int j = 0; j < KP; ++j)
            r.blk[i * KP + j] = b.val * a.blk[i * KP + j] + a.grad[i] * b.grad[KX + j]
                              + b.grad[i] * a.grad[KX + j] + a.val * b.blk[i * KP + j];
    return r;
}
TAD_TPL TAD_HD TAD_M operator/(const TAD_M& a, const TAD_M& b)
{
    TAD_M r;
    const T ib = T(1) / b.val;
    r.val = a.val * ib;
#pragma unroll
    for (int i = 0; i < KX + KP; ++i) r.grad[i] = (a.grad[i] - r.val * b.grad[i]) * ib;
#pragma unroll
    for (int i = 0; i < KX; ++i)
#pragma unroll
        for (int j = 0; j < KP; ++j)
            r.blk[i * KP + j] = (a.blk[i * KP + j] - r.grad[i] * b.grad[KX + j] - b.grad[i] * r.grad[KX + j]
                                 - r.val * b.blk[i * KP + j]) * ib;
    return r;
}
TAD_TPLU TAD_HD TAD_M operator*(const TAD_M& a, U s)
{
    TAD_M r; const T t = T(s); r.val = a.val * t;
#pragma unroll
    for (int i = 0; i < KX + KP; ++i) r.grad[i] = a.grad[i] * t;
#pragma unroll
    for (int i = 0; i < KX * KP; ++i) r.blk[i] = a.blk[i] * t;
    return r;
}
TAD_TPLU TAD_HD TAD_M operator*(U s, const TAD_M& a) { return a * s; }
TAD_TPLU TAD_HD TAD_M operator+(const TAD_M& a, U s) { TAD_M r = a; r.val += T(s); return r; }
TAD_TPLU TAD_HD TAD_M operator-(const TAD_M& a, U s) { TAD_M r = a; r.val -= T(s); return r; }
TAD_TPLU TAD_HD TAD_M operator/(U c, const TAD_M& b) { const TAD_M one{T(c)}; return one / b; }
TAD_TPLU TAD_HD TAD_M operator/(const TAD_M& a, U s) { return a * (T(1) / T(s)); }
TAD_TPL TAD_HD TAD_M sqrt(const TAD_M& a)
{
    using std::sqrt;
    const T f = sqrt(a.val);
    return TAD_M::chain(f, T(0.5) / f, T(-0.25) / (f * a.val), a);
}
TAD_TPL TAD_HD TAD_M sqr(const TAD_M& a) { return a * a; }
TAD_TPLU TAD_HD TAD_M operator+(U s, const TAD_M& a) { return a + s; }
TAD_TPLU TAD_HD TAD_M operator-(U s, const TAD_M& a) { return (-a) + s; }
TAD_TPLU TAD_HD bool operator<=(const TAD_M& a, U b) { return a.val <= T(b); }
TAD_TPL TAD_HD T to_passive(const TAD_M& a) { return a.val; }
#undef TAD_TPLU
#undef TAD_TPL
#undef TAD_M

} // namespace tad
