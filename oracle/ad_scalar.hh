/*
 * ORACLE -- test infrastructure only.  Not part of the product.
 *
 * Dense forward-mode second-order scalar: a CPU restatement of TinyAD's
 * Scalar<k, PassiveT, with_hessian, r0, c0, rows, cols>
 * (include/TinyAD/Scalar.hh:24-1347).  The Hessian is stored full and dense
 * (column-major, like the reference's Eigen matrix), optionally restricted
 * to the block [R0, R0+NR) x [C0, C0+NC) (Scalar.hh:24, :186-196).
 * Each operator follows the reference formula and evaluation order cited
 * beside it.  Only the tests, the bench's CPU-baseline leg and the oracle's
 * own C ABI use this file.
 */
#pragma once
#include <cmath>
#include <array>

namespace oracle {

template <int K, typename T, int R0 = 0, int C0 = 0, int NR = K, int NC = K>
struct AD
{
    static constexpr int k = K;
    static constexpr bool truncated = (R0 != 0 || C0 != 0 || NR != K || NC != K);
    T val = 0;
    std::array<T, K> grad{};
    std::array<T, (NR * NC > 0 ? NR * NC : 1)> hess{};   // column-major NR x NC

    AD() = default;
    AD(T v) : val(v) {}                                   // passive (Scalar.hh:58-63)
    AD(T v, int idx) : val(v) { grad[idx] = T(1); }      // active (Scalar.hh:67-75)

    T& H(int i, int j) { return hess[j * NR + i]; }
    const T& H(int i, int j) const { return hess[j * NR + i]; }

    static AD known(T v, T g, T h)                        // Scalar.hh:89-101 (k == 1)
    {
        AD r; r.val = v; r.grad[0] = g; if (NR * NC > 0) r.hess[0] = h; return r;
    }

    // outer(ga, gb) restricted to the Hessian block (Scalar.hh:186-196)
    static T outer(const std::array<T, K>& ga, const std::array<T, K>& gb, int i, int j)
    {
        return ga[R0 + i] * gb[C0 + j];
    }

    // chain rule f(a): val, df/da, d2f/da2 (Scalar.hh:199-214):
    // Hess = Hess_f * outer(ga, ga) + grad_f * a.Hess
    static AD chain(T f, T f1, T f2, const AD& a)
    {
        AD r; r.val = f;
        for (int i = 0; i < K; ++i) r.grad[i] = f1 * a.grad[i];
        for (int j = 0; j < NC; ++j)
            for (int i = 0; i < NR; ++i)
                r.H(i, j) = f2 * outer(a.grad, a.grad, i, j) + f1 * a.H(i, j);
        return r;
    }
};

template <typename S> using PT = decltype(S::val);

// ---- unary ---------------------------------------------------------------
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator-(const AD<K, T, R0, C0, NR, NC>& a)       // Scalar.hh:220-234
{
    AD<K, T, R0, C0, NR, NC> r; r.val = -a.val;
    for (int i = 0; i < K; ++i) r.grad[i] = -a.grad[i];
    for (size_t i = 0; i < r.hess.size(); ++i) r.hess[i] = -a.hess[i];
    return r;
}

template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> sqrt(const AD<K, T, R0, C0, NR, NC>& a)            // Scalar.hh:236-247
{
    const T f = std::sqrt(a.val);
    return AD<K, T, R0, C0, NR, NC>::chain(f, T(0.5) / f, T(-0.25) / (f * a.val), a);
}

template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> sqr(const AD<K, T, R0, C0, NR, NC>& a)             // Scalar.hh:249-264
{
    AD<K, T, R0, C0, NR, NC> r; r.val = a.val * a.val;
    for (int i = 0; i < K; ++i) r.grad[i] = T(2) * a.val * a.grad[i];
    for (int j = 0; j < NC; ++j)
        for (int i = 0; i < NR; ++i)
            r.H(i, j) = T(2) * (a.val * a.H(i, j) + AD<K, T, R0, C0, NR, NC>::outer(a.grad, a.grad, i, j));
    return r;
}

template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> pow(const AD<K, T, R0, C0, NR, NC>& a, int e)      // Scalar.hh:266-289
{
    using S = AD<K, T, R0, C0, NR, NC>;
    if (e == 0) return S::chain(T(1), T(0), T(0), a);
    if (e == 1) return S::chain(a.val, T(1), T(0), a);
    const T f2 = (T)std::pow(a.val, e - 2);
    const T f1 = f2 * a.val;
    const T f = f1 * a.val;
    return S::chain(f, e * f1, e * (e - 1) * f2, a);
}

template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> pow(const AD<K, T, R0, C0, NR, NC>& a, T e)        // Scalar.hh:291-307
{
    const T f2 = std::pow(a.val, e - T(2));
    const T f1 = f2 * a.val;
    const T f = f1 * a.val;
    return AD<K, T, R0, C0, NR, NC>::chain(f, e * f1, e * (e - T(1)) * f2, a);
}

#define ORACLE_UNARY(NAME, ...)                                                  \
template <int K, typename T, int R0, int C0, int NR, int NC>                    \
AD<K, T, R0, C0, NR, NC> NAME(const AD<K, T, R0, C0, NR, NC>& a)                \
{ using S = AD<K, T, R0, C0, NR, NC>; const T v = a.val; __VA_ARGS__ }

ORACLE_UNARY(exp,  { const T e = std::exp(v); return S::chain(e, e, e, a); })                   // Scalar.hh:324-332
ORACLE_UNARY(log,  { const T ai = T(1) / v; return S::chain(std::log(v), ai, -ai / v, a); })     // Scalar.hh:334-346
ORACLE_UNARY(sin,  { const T s = std::sin(v); return S::chain(s, std::cos(v), -s, a); })         // Scalar.hh:374-385
ORACLE_UNARY(cos,  { const T c = std::cos(v); return S::chain(c, -std::sin(v), -c, a); })        // Scalar.hh:387-398
ORACLE_UNARY(tan,  { const T c = std::cos(v); const T c2 = c * c; const T c3 = c2 * c;
                     return S::chain(std::tan(v), T(1) / c2, T(2) * std::sin(v) / c3, a); })     // Scalar.hh:400-413
ORACLE_UNARY(asin, { const T s = T(1) - v * v; const T ss = std::sqrt(s);
                     return S::chain(std::asin(v), T(1) / ss, v / ss / s, a); })                 // Scalar.hh:415-426
ORACLE_UNARY(acos, { const T s = T(1) - v * v; const T ss = std::sqrt(s);
                     return S::chain(std::acos(v), T(-1) / ss, -v / ss / s, a); })               // Scalar.hh:428-446
ORACLE_UNARY(atan, { const T s = v * v + T(1);
                     return S::chain(std::atan(v), T(1) / s, T(-2) * v / s / s, a); })           // Scalar.hh:448-458
ORACLE_UNARY(sinh, { const T s = std::sinh(v); return S::chain(s, std::cosh(v), s, a); })        // Scalar.hh:460-471
ORACLE_UNARY(cosh, { const T c = std::cosh(v); return S::chain(c, std::sinh(v), c, a); })        // Scalar.hh:473-484
ORACLE_UNARY(tanh, { const T c = std::cosh(v); const T c2 = c * c; const T c3 = c2 * c;
                     return S::chain(std::tanh(v), T(1) / c2, T(-2) * std::sinh(v) / c3, a); }) // Scalar.hh:486-499
ORACLE_UNARY(log2, { const T ai = T(1) / v / T(std::log(2.0)); return S::chain(std::log2(v), ai, -ai / v, a); })   // Scalar.hh:348-358
ORACLE_UNARY(log10,{ const T ai = T(1) / v / T(std::log(10.0)); return S::chain(std::log10(v), ai, -ai / v, a); }) // Scalar.hh:360-370
ORACLE_UNARY(asinh,{ const T s = v * v + T(1); const T ss = std::sqrt(s);
                     return S::chain(std::asinh(v), T(1) / ss, -v / ss / s, a); })                 // Scalar.hh:501-515
ORACLE_UNARY(acosh,{ const T sm = v - T(1), sp = v + T(1); const T pr = std::sqrt(sm) * std::sqrt(sp);
                     return S::chain(std::acosh(v), T(1) / pr, -v / pr / sm / sp, a); })           // Scalar.hh:517-534
ORACLE_UNARY(atanh,{ const T s = T(1) - v * v;
                     return S::chain(std::atanh(v), T(1) / s, T(2) * v / s / s, a); })             // Scalar.hh:536-546
ORACLE_UNARY(fabs, { return v >= T(0) ? S::chain(v, T(1), T(0), a) : S::chain(-v, T(-1), T(0), a); }) // Scalar.hh:309-322
#undef ORACLE_UNARY

// ---- binary --------------------------------------------------------------
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator+(const AD<K, T, R0, C0, NR, NC>& a, const AD<K, T, R0, C0, NR, NC>& b)  // Scalar.hh:579-595
{
    AD<K, T, R0, C0, NR, NC> r; r.val = a.val + b.val;
    for (int i = 0; i < K; ++i) r.grad[i] = a.grad[i] + b.grad[i];
    for (size_t i = 0; i < r.hess.size(); ++i) r.hess[i] = a.hess[i] + b.hess[i];
    return r;
}
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator+(const AD<K, T, R0, C0, NR, NC>& a, T b) { auto r = a; r.val += b; return r; }  // :597-608
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator+(T a, const AD<K, T, R0, C0, NR, NC>& b) { auto r = b; r.val += a; return r; }  // :610-621

template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator-(const AD<K, T, R0, C0, NR, NC>& a, const AD<K, T, R0, C0, NR, NC>& b)  // Scalar.hh:651-667
{
    AD<K, T, R0, C0, NR, NC> r; r.val = a.val - b.val;
    for (int i = 0; i < K; ++i) r.grad[i] = a.grad[i] - b.grad[i];
    for (size_t i = 0; i < r.hess.size(); ++i) r.hess[i] = a.hess[i] - b.hess[i];
    return r;
}
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator-(const AD<K, T, R0, C0, NR, NC>& a, T b) { auto r = a; r.val -= b; return r; }  // :669-680
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator-(T a, const AD<K, T, R0, C0, NR, NC>& b)                                      // :682-698
{
    AD<K, T, R0, C0, NR, NC> r; r.val = a - b.val;
    for (int i = 0; i < K; ++i) r.grad[i] = -b.grad[i];
    for (size_t i = 0; i < r.hess.size(); ++i) r.hess[i] = -b.hess[i];
    return r;
}

// a*b: Hess = b.val*Ha + outer(ga,gb) + outer(gb,ga) + a.val*Hb (Scalar.hh:738-769)
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator*(const AD<K, T, R0, C0, NR, NC>& a, const AD<K, T, R0, C0, NR, NC>& b)
{
    using S = AD<K, T, R0, C0, NR, NC>;
    S r; r.val = a.val * b.val;
    for (int i = 0; i < K; ++i) r.grad[i] = b.val * a.grad[i] + a.val * b.grad[i];
    for (int j = 0; j < NC; ++j)
        for (int i = 0; i < NR; ++i)
            r.H(i, j) = ((b.val * a.H(i, j) + S::outer(a.grad, b.grad, i, j)) + S::outer(b.grad, a.grad, i, j)) + a.val * b.H(i, j);
    return r;
}
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator*(const AD<K, T, R0, C0, NR, NC>& a, T b)                                      // :771-786
{
    auto r = a; r.val *= b;
    for (auto& v : r.grad) v *= b;
    for (auto& v : r.hess) v *= b;
    return r;
}
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator*(T a, const AD<K, T, R0, C0, NR, NC>& b) { return b * a; }                    // :788-803

// a/b (Scalar.hh:823-840):
//   grad = (b.val*ga - a.val*gb) / (b.val^2)
//   Hess = (Ha - outer(g_r, gb) - outer(gb, g_r) - r*Hb) / b.val
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator/(const AD<K, T, R0, C0, NR, NC>& a, const AD<K, T, R0, C0, NR, NC>& b)
{
    using S = AD<K, T, R0, C0, NR, NC>;
    S r; r.val = a.val / b.val;
    const T bb = b.val * b.val;
    for (int i = 0; i < K; ++i) r.grad[i] = (b.val * a.grad[i] - a.val * b.grad[i]) / bb;
    for (int j = 0; j < NC; ++j)
        for (int i = 0; i < NR; ++i)
            r.H(i, j) = (((a.H(i, j) - S::outer(r.grad, b.grad, i, j)) - S::outer(b.grad, r.grad, i, j)) - r.val * b.H(i, j)) / b.val;
    return r;
}
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator/(const AD<K, T, R0, C0, NR, NC>& a, T b)                                      // :842-857
{
    auto r = a; r.val /= b;
    for (auto& v : r.grad) v /= b;
    for (auto& v : r.hess) v /= b;
    return r;
}
// a/b with passive a (Scalar.hh:859-877):
//   grad = (-a / b.val^2) * gb ; Hess = (outer(-g_r, gb) - outer(gb, g_r) - r*Hb) / b.val
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> operator/(T a, const AD<K, T, R0, C0, NR, NC>& b)
{
    using S = AD<K, T, R0, C0, NR, NC>;
    S r; r.val = a / b.val;
    const T c = -a / (b.val * b.val);
    for (int i = 0; i < K; ++i) r.grad[i] = c * b.grad[i];
    std::array<T, K> mg; for (int i = 0; i < K; ++i) mg[i] = -r.grad[i];
    for (int j = 0; j < NC; ++j)
        for (int i = 0; i < NR; ++i)
            r.H(i, j) = ((S::outer(mg, b.grad, i, j) - S::outer(b.grad, r.grad, i, j)) - r.val * b.H(i, j)) / b.val;
    return r;
}

// atan2 (Scalar.hh:891-915)
template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> atan2(const AD<K, T, R0, C0, NR, NC>& y, const AD<K, T, R0, C0, NR, NC>& x)
{
    using S = AD<K, T, R0, C0, NR, NC>;
    S r; r.val = std::atan2(y.val, x.val);
    std::array<T, K> u, dv;
    for (int i = 0; i < K; ++i) u[i] = x.val * y.grad[i] - y.val * x.grad[i];
    const T v = x.val * x.val + y.val * y.val;
    for (int i = 0; i < K; ++i) r.grad[i] = u[i] / v;
    for (int i = 0; i < K; ++i) dv[i] = T(2) * (x.val * x.grad[i] + y.val * y.grad[i]);
    for (int j = 0; j < NC; ++j)
        for (int i = 0; i < NR; ++i)
        {
            const T du = ((x.val * y.H(i, j) - y.val * x.H(i, j)) + S::outer(y.grad, x.grad, i, j)) - S::outer(x.grad, y.grad, i, j);
            r.H(i, j) = (du - r.grad[R0 + i] * dv[C0 + j]) / v;
        }
    return r;
}

template <int K, typename T, int R0, int C0, int NR, int NC>
AD<K, T, R0, C0, NR, NC> hypot(const AD<K, T, R0, C0, NR, NC>& a, const AD<K, T, R0, C0, NR, NC>& b)  // :917-926
{
    return sqrt(a * a + b * b);
}

// comparisons on .val only (Scalar.hh:933-1095)
template <int K, typename T, int R0, int C0, int NR, int NC>
bool operator<=(const AD<K, T, R0, C0, NR, NC>& a, T b) { return a.val <= b; }
template <int K, typename T, int R0, int C0, int NR, int NC>
bool operator<(const AD<K, T, R0, C0, NR, NC>& a, T b) { return a.val < b; }

inline double value_of(double v) { return v; }
inline float value_of(float v) { return v; }
template <int K, typename T, int R0, int C0, int NR, int NC>
T value_of(const AD<K, T, R0, C0, NR, NC>& a) { return a.val; }

} // namespace oracle
