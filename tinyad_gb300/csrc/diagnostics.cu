/*
 * tad_debug_scalar_op: runs one tad::Scalar<1> operator on the device so the
 * operator known-answer tests of the reference (tests/ScalarTestUnary
 * Operators.cc, tests/ScalarTestBinaryOperators.cc) can be checked against
 * the device type.  Op codes are listed in include/tad.h.
 */
#include "internal.hh"
#include "../../include/tad/Scalar.cuh"

namespace tadlib {

template <typename S>
__device__ S apply_op(int op, const S& a, const S& b, double bv)
{
    using V = typename S::passive_type;
    switch (op)
    {
    case 0: return -a;
    case 1: return tad::sqrt(a);
    case 2: return tad::sqr(a);
    case 3: return tad::pow(a, (int)bv);
    case 4: return tad::pow(a, (V)bv);
    case 5: return tad::exp(a);
    case 6: return tad::log(a);
    case 7: return tad::sin(a);
    case 8: return tad::cos(a);
    case 9: return tad::tan(a);
    case 10: return tad::asin(a);
    case 11: return tad::acos(a);
    case 12: return tad::atan(a);
    case 13: return tad::sinh(a);
    case 14: return tad::cosh(a);
    case 15: return tad::tanh(a);
    case 16: return tad::fabs(a);
    case 17: return a + b;
    case 18: return a - b;
    case 19: return a * b;
    case 20: return a / b;
    case 21: return tad::atan2(a, b);
    case 22: return tad::hypot(a, b);
    case 23: return (V)bv / a;
    case 24: return tad::log2(a);
    case 25: return tad::log10(a);
    case 26: return tad::asinh(a);
    case 27: return tad::acosh(a);
    case 28: return tad::atanh(a);
    case 29: return a + (V)bv;
    case 30: return a * (V)bv;
    case 31: return (V)bv - a;
    case 32: return a / (V)bv;
    }
    return S(V(0));
}

template <typename S>
__global__ void k_scalar_op(int op, double a0, double a1, double a2, double b0, double b1, double b2, double* out)
{
    using T = typename S::deriv_type;
    using G = typename S::grad_type;
    const S a = S::known_derivatives(a0, (G)a1, (T)a2);
    const S b = S::known_derivatives(b0, (G)b1, (T)b2);
    const S r = apply_op<S>(op, a, b, b0);
    out[0] = (double)r.val;
    out[1] = (double)r.grad[0];
    out[2] = (double)r.hess[0];
}

} // namespace tadlib

using namespace tadlib;

extern "C" TAD_API tad_status tad_debug_scalar_op(int op, int precision, const double* a3, const double* b3, double* out3)
{
    if (op < 0 || op > 32 || !a3 || !b3 || !out3) { set_error("bad argument"); return TAD_ERR_ARG; }
    double* d = nullptr;
    TAD_CUDA_TRY(cudaMalloc(&d, 3 * sizeof(double)));
    if (precision == TAD_PREC_MIXED)
        k_scalar_op<tad::Mixed<1>><<<1, 1>>>(op, a3[0], a3[1], a3[2], b3[0], b3[1], b3[2], d);
    else
        k_scalar_op<tad::Double<1>><<<1, 1>>>(op, a3[0], a3[1], a3[2], b3[0], b3[1], b3[2], d);
    cudaError_t e = cudaMemcpy(out3, d, 3 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d);
    TAD_CUDA_TRY(e);
    return TAD_OK;
}

/* ------------------------------------------------------------------------ */
/* CUDA-core FMA throughput (roofline denominators for element evaluation): */
/* 8 independent FMA chains per thread, grid = 8 x SMs blocks of 256.       */
/* ------------------------------------------------------------------------ */
namespace tadlib {
template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T seed, T* out)
{
    T a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = seed + T(i) * T(1e-3) + T(threadIdx.x) * T(1e-7);
    const T m = T(0.999999), c = T(1e-7);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = a[i] * m + c;
    T s = T(0);
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == T(-12345.0)) out[0] = s;   // keeps the chains live
}
} // namespace tadlib

extern "C" TAD_API tad_status tad_measure_fma_peak(int precision, double* tflops)
{
    if (!tflops) { set_error("NULL argument"); return TAD_ERR_ARG; }
    int dev = 0, sms = 0;
    TAD_CUDA_TRY(cudaGetDevice(&dev));
    TAD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    TAD_CUDA_TRY(cudaMalloc(&out, 8));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    const int iters = precision == TAD_PREC_MIXED ? 4096 : 256;
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep)
    {
        cudaEventRecord(e0);
        if (precision == TAD_PREC_MIXED) k_fma_peak<float><<<blocks, threads>>>(iters, 1.0f, (float*)out);
        else k_fma_peak<double><<<blocks, threads>>>(iters, 1.0, out);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    TAD_CUDA_TRY(cudaGetLastError());
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return TAD_OK;
}
