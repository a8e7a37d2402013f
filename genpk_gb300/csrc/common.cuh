// common.cuh -- device helpers shared by the deposit, binning and adjoint kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace genpk {

// Position -> (wrapped cell, fraction) for one axis, as fieldize.cpp:66-76
// computes it in FP64: x = pos*units, f = floor(x), d = x - f, f wrapped mod N.
//
// units = dims/boxsize is carried as an unevaluated float sum hi + lo, and the
// product pos*units is formed exactly as xh + xl with one FMA (Dekker's
// two-product), so d is accurate to ~1e-7 of a cell even where a plain FP32
// product of a box-sized coordinate is only good to ~3e-5 of a cell.  The
// integer part comes from xh; the carry into or out of [0,1) is fixed up.
__device__ __forceinline__ void split_cell(float p, float uh, float ul, int dims, int &cell,
                                           float &frac)
{
    const float xh = __fmul_rn(p, uh);
    const float xe = fmaf(p, uh, -xh);  // exact rounding error of p*uh
    const float xl = fmaf(p, ul, xe);
    const float f = floorf(xh);
    float d = __fadd_rn(__fsub_rn(xh, f), xl);
    int fi = (int)f;
    if (d < 0.f) {
        d = __fadd_rn(d, 1.f);
        fi -= 1;
    }
    if (d >= 1.f) {
        d = __fsub_rn(d, 1.f);
        fi += 1;
    }
    if ((unsigned)fi >= (unsigned)dims) {  // outside [0, dims): periodic wrap
        fi %= dims;
        if (fi < 0)
            fi += dims;
    }
    cell = fi;
    frac = d;
}

// Nearest float to a 64-bit integer (ties to even), with integer instructions
// only: the hardware int64 -> float conversion runs on the FP64 pipe, which
// GB300 has little of.
__device__ __forceinline__ float i64_to_f32_rn(long long v)
{
    const unsigned neg = (unsigned)((unsigned long long)v >> 63);
    unsigned long long a = neg ? 0ull - (unsigned long long)v : (unsigned long long)v;
    if (a == 0ull)
        return 0.f;
    int e = 63 - __clzll((long long)a);  // position of the leading one
    unsigned m;
    if (e <= 23) {
        m = (unsigned)a << (23 - e);
    } else {
        const int sh = e - 23;
        unsigned long long q = a >> sh;
        const unsigned long long rem = a & ((1ull << sh) - 1ull);
        const unsigned long long half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (q & 1ull)))
            q++;
        if (q == (1ull << 24)) {
            q >>= 1;
            e++;
        }
        m = (unsigned)q;
    }
    return __uint_as_float((neg << 31) | ((unsigned)(e + 127) << 23) | (m & 0x7fffffu));
}

// Unevaluated sum hi + lo of two floats (double-float arithmetic, Dekker/Knuth).
struct f2sum {
    float hi, lo;
};

__device__ __forceinline__ f2sum two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ f2sum renorm(float hi, float lo)
{
    const float s = __fadd_rn(hi, lo);
    return {s, __fsub_rn(lo, __fsub_rn(s, hi))};
}

__device__ __forceinline__ f2sum f2_add(f2sum a, float b)
{
    const f2sum s = two_sum(a.hi, b);
    return renorm(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ f2sum f2_add2(f2sum a, f2sum b)
{
    const f2sum s = two_sum(a.hi, b.hi);
    return renorm(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ f2sum f2_mul(f2sum a, f2sum b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return renorm(p, e);
}

// 1 - 2d for one axis of a particle, d = x - floor(x), x = p*units, as a float
// pair good to ~2^-44.  The carry decisions repeat split_cell's exactly, so the
// value belongs to the same cell split_cell returns.
__device__ __forceinline__ f2sum one_minus_2frac(float p, float uh, float ul)
{
    const float xh = __fmul_rn(p, uh);
    const float xe = fmaf(p, uh, -xh);
    const float xl = fmaf(p, ul, xe);
    const float f = floorf(xh);
    f2sum d = two_sum(__fsub_rn(xh, f), xl);
    if (d.hi < 0.f)
        d = f2_add(d, 1.f);
    if (d.hi >= 1.f)
        d = f2_add(d, -1.f);
    const f2sum u = two_sum(1.f, -2.f * d.hi);
    return renorm(u.hi, __fsub_rn(u.lo, 2.f * d.lo));
}

// One axis of a particle in full: the wrapped cell and FP32 fraction exactly as
// split_cell computes them, plus what the exact corner-mode term needs:
// u = 1 - 2*(xh - floor) for the final cell (exact in FP32 for xh >= 1; one
// rounding below) and xl, the low part of x = xh + xl, so that
// 1 - 2d = u - 2*xl exactly.
struct AxisSplit {
    int cell;
    float frac;
    float u;
    float xl;
};

__device__ __forceinline__ AxisSplit split_axis(float p, float uh, float ul, int dims)
{
    const float xh = __fmul_rn(p, uh);
    const float xe = fmaf(p, uh, -xh);
    const float xl = fmaf(p, ul, xe);
    const float f = floorf(xh);
    const float a = __fsub_rn(xh, f);
    float d = __fadd_rn(a, xl);
    float u = fmaf(-2.f, a, 1.f);
    int fi = (int)f;
    if (d < 0.f) {
        d = __fadd_rn(d, 1.f);
        fi -= 1;
        u = __fsub_rn(u, 2.f);
    }
    if (d >= 1.f) {
        d = __fsub_rn(d, 1.f);
        fi += 1;
        u = __fadd_rn(u, 2.f);
    }
    if ((unsigned)fi >= (unsigned)dims) {
        fi %= dims;
        if (fi < 0)
            fi += dims;
    }
    return {fi, d, u, xl};
}

// prod_a (1 - 2 d_a) = prod_a (u_a - 2 xl_a) as a float pair: the product of
// the u's with two-product steps (error ~2^-47) plus the first-order xl terms
// in FP32 (second-order terms are ~2^-48 and dropped).
__device__ __forceinline__ f2sum corner_factor(const AxisSplit &x, const AxisSplit &y,
                                               const AxisSplit &z)
{
    const float p = __fmul_rn(x.u, y.u);
    const float pl = fmaf(x.u, y.u, -p);
    const float q = __fmul_rn(p, z.u);
    const float ql = fmaf(p, z.u, -q) + pl * z.u;
    const float corr = -2.f * (x.xl * (y.u * z.u) + y.xl * (x.u * z.u) + z.xl * (x.u * y.u));
    return {q, ql + corr};
}

// 24-bit fixed point of a fraction in [0,1); exact in FP32 on the way back.
__device__ __forceinline__ uint32_t frac_to_q24(float d)
{
    uint32_t q = (uint32_t)(d * 16777216.f);
    return q > 0xFFFFFFu ? 0xFFFFFFu : q;
}

__device__ __forceinline__ float q24_to_frac(uint32_t w)
{
    return (float)(w & 0xFFFFFFu) * (1.f / 16777216.f);
}

__device__ __forceinline__ bool finite3(float a, float b, float c)
{
    return isfinite(a) && isfinite(b) && isfinite(c);
}

// Index of the float at cell (x, y, z) of the padded grid.
__device__ __forceinline__ size_t cell_index(int64_t plane, int row, int x, int y, int z)
{
    return (size_t)x * (size_t)plane + (size_t)y * (size_t)row + (size_t)z;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace genpk
