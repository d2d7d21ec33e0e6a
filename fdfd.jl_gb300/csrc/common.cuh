// Shared device/host definitions for libfdfd_cuda.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

// ---- device error word bits (OR-ed by kernels, read by the host) ----------
#define FDFD_DEVERR_SINGULAR 1u
#define FDFD_DEVERR_TIMEOUT  2u
#define FDFD_DEVERR_NONFINITE 4u

// ---- complex helpers -------------------------------------------------------
template <typename T> struct cplx { T re, im; };

template <typename T> __host__ __device__ __forceinline__ cplx<T> cmk(T r, T i) { cplx<T> z; z.re = r; z.im = i; return z; }
template <typename T> __host__ __device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) { return cmk(a.re + b.re, a.im + b.im); }
template <typename T> __host__ __device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) { return cmk(a.re - b.re, a.im - b.im); }
template <typename T> __host__ __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> cscale(cplx<T> a, T s) { return cmk(a.re * s, a.im * s); }
template <typename T> __host__ __device__ __forceinline__ cplx<T> cneg(cplx<T> a) { return cmk(-a.re, -a.im); }
// 1/z by Smith's algorithm (R. L. Smith, CACM 5(8), 1962), avoids overflow.
template <typename T> __host__ __device__ __forceinline__ cplx<T> cinv(cplx<T> z) {
    T a = z.re, b = z.im;
    if (fabs(a) >= fabs(b)) {
        T r = b / a, d = a + b * r;
        return cmk((T)1 / d, -r / d);
    } else {
        T r = a / b, d = a * r + b;
        return cmk(r / d, (T)-1 / d);
    }
}
template <typename T> __host__ __device__ __forceinline__ T cabs1(cplx<T> a) { return fabs(a.re) + fabs(a.im); }
// acc ± c·v in four FMAs (the negations are free operand modifiers).  The FP64
// vector and stencil kernels are bound by FP64 issue on this part, not by HBM.
template <bool kSub, typename T>
__device__ __forceinline__ void cmac(cplx<T>& acc, cplx<T> c, cplx<T> v) {
    if (kSub) {
        acc.re = fma(-c.re, v.re, acc.re);
        acc.re = fma(c.im, v.im, acc.re);
        acc.im = fma(-c.re, v.im, acc.im);
        acc.im = fma(-c.im, v.re, acc.im);
    } else {
        acc.re = fma(c.re, v.re, acc.re);
        acc.re = fma(-c.im, v.im, acc.re);
        acc.im = fma(c.re, v.im, acc.im);
        acc.im = fma(c.im, v.re, acc.im);
    }
}

// ---- FP64 arithmetic without FMA contraction (mirrors Julia's rounding) ----
__device__ __forceinline__ cplx<double> cmul_rn(cplx<double> a, cplx<double> b) {
    return cmk(__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
               __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re)));
}
__device__ __forceinline__ cplx<double> cadd_rn(cplx<double> a, cplx<double> b) {
    return cmk(__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im));
}
__device__ __forceinline__ cplx<double> cscale_rn(cplx<double> a, double s) {
    return cmk(__dmul_rn(a.re, s), __dmul_rn(a.im, s));
}

// ---- TF32 split: x = hi + lo with hi the top 19 bits of x (sign, exponent,
// 10 mantissa bits) and lo = x - hi exact in FP32. ---------------------------
__device__ __forceinline__ float tf32_lo(float x) {
    float hi = __uint_as_float(__float_as_uint(x) & 0xffffe000u);
    return x - hi;
}

// ---- block pools -----------------------------------------------------------
// A pool holds `count` complex matrices of `rows` x `cols` (row-major, leading
// dimension `ld`).  Each slot stores `planes` real planes of rows*ld values:
// plane 0 = real part, 1 = imaginary part and, for the FP32 Gauss-Jordan panel
// buffers only, 2/3 = the TF32 residuals (lo) of planes 0/1 (pre-split
// tensor-core operands).
template <typename T> struct Pool {
    T* base = nullptr;
    int rows = 0, cols = 0, ld = 0, planes = 2;
    long long count = 0;
    __host__ __device__ long long plane_elems() const { return (long long)rows * ld; }
    __host__ __device__ long long slot_elems() const { return plane_elems() * planes; }
    __host__ __device__ T* slot(long long s) const { return base + s * slot_elems(); }
};

// ---- bounded waits ---------------------------------------------------------
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
#define FDFD_WAIT_LIMIT_NS 2000000000ull  // 2 s

__device__ __forceinline__ void dev_error(unsigned* err, unsigned bits) {
    if (err) atomicOr(err, bits);
}

// ---- mbarriers (shared memory) ---------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false once limit_ns of %globaltimer have passed.  The tensor-core
// GEMM's pipeline waits take the launch's limit (GemmArgs::wait_ns, settable per
// handle); the waits that drain a CTA's own copies and MMAs in flight before it
// frees TMEM and exits always take FDFD_WAIT_LIMIT_NS, so a short pipeline limit
// never lets a CTA leave with asynchronous work outstanding.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try(bar, parity)) return true;
    uint64_t t0 = globaltimer_ns();
    while (true) {
        if (mbar_try(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit_ns) return false;
        __nanosleep(64);
    }
}
// the same bound without the back-off, for waits expected to end within a few
// hundred cycles
__device__ __forceinline__ bool mbar_wait_spin(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try(bar, parity))
        if (globaltimer_ns() - t0 > limit_ns) return false;
    return true;
}

// ---- misc ------------------------------------------------------------------
static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
