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

// Nearest float to a 64-bit integer (ties to even) from 32-bit operations:
// the hardware int64 -> float conversion runs on the FP64 pipe, which GB300
// has little of.  |v| < 2^32 converts directly (32-bit conversion, nearest
// even); above, the top 32 bits of |v| from its leading one, with every lower
// bit ORed into bit 0 (a sticky bit below the rounding position, bit 7), round
// the same way and are scaled back by an exact power of two.
__device__ __forceinline__ float i64_to_f32_rn(long long v)
{
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    const unsigned hi = (unsigned)(a >> 32), lo = (unsigned)a;
    float r;
    if (hi == 0u) {
        r = __uint2float_rn(lo);
    } else {
        const int k = __clz((int)hi);                      // hi << k has bit 31 set
        const unsigned top = __funnelshift_l(lo, hi, k);   // bits 63-k .. 32-k of |v|
        const unsigned sticky = (lo << k) != 0u ? 1u : 0u;  // the 32-k bits below
        r = __uint2float_rn(top | sticky) * __uint_as_float((unsigned)(159 - k) << 23);  // 2^(32-k)
    }
    return v < 0 ? -r : r;
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

// acc += v for a running sum kept as an unnormalised pair: hi is the rounded
// sum of the high parts, lo collects their exact rounding errors and the low
// parts (the pair is renormalised only when sums are combined at the end).
__device__ __forceinline__ void f2_accumulate(f2sum &acc, f2sum v)
{
    const f2sum s = two_sum(acc.hi, v.hi);
    acc.hi = s.hi;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, v.lo));
}

// v * (-1)^parity (sign flips of both parts; parity in bit 0).
__device__ __forceinline__ f2sum f2_signed(f2sum v, int parity)
{
    const unsigned flip = (unsigned)parity << 31;
    return {__uint_as_float(__float_as_uint(v.hi) ^ flip),
            __uint_as_float(__float_as_uint(v.lo) ^ flip)};
}

__device__ __forceinline__ f2sum f2_mul(f2sum a, f2sum b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return renorm(p, e);
}

// One axis split to a 28-bit fixed-point fraction, from the exact two-product
// x = xh + xl (no FP32 rounding of the fraction): q = round((xh - floor(xh) +
// xl) * 2^28) with at most 2^-28 error, the cell moved when the carry leaves
// [0, 1).  u = 1 - 2*(xh - floor) (moved with the cell) and xl feed the exact
// corner-mode term (1 - 2d = u - 2 xl exactly).  FP32 fractions are not enough: a smooth
// lattice's faintest high-k bins moved by 2.5e-5 with FP32 fractions and by
// 2.5e-7 with 32-bit ones in an emulation at 128^3.
struct AxisQ {
    int cell;
    uint32_t q;  // fraction * 2^28, in [0, 2^28)
    float u;
    float xl;
};

constexpr int kFracBits = 28;
constexpr uint32_t kFracOne = 1u << kFracBits;

__device__ __forceinline__ AxisQ split_q28(float p, float uh, float ul, int dims)
{
    const float xh = __fmul_rn(p, uh);
    const float xe = fmaf(p, uh, -xh);
    float xl = fmaf(p, ul, xe);
    const float f = floorf(xh);
    float a = __fsub_rn(xh, f);
    // For |xh| >= 1, a is exact and a multiple of 2^-23, so 1 - 2a is exact.
    // Within one cell of the origin both may round (a = xh + 1 for
    // -1 < xh < 0; 1 - 2a for a < 1/4): the errors move into xl, so that the
    // fraction a + xl and u - 2 xl (the corner factor) stay exact.
    float u = fmaf(-2.f, a, 1.f);
    float xlu = xl;
    if (fabsf(xh) < 1.f) {
        const f2sum s = two_sum(xh, -f);
        a = s.hi;
        xl = __fadd_rn(xl, s.lo);
        const f2sum t = two_sum(1.f, -2.f * a);
        u = t.hi;
        xlu = __fsub_rn(xl, 0.5f * t.lo);
    }
    // a * 2^28 is exact (an integer when xh >= 1); xl * 2^28 is at most
    // ~|x| 2^5, clamped so that the sum cannot overflow (exact up to 2^25 cells)
    const int qa = __float2int_rn(a * 268435456.f);
    const int qb = min(max(__float2int_rn(xl * 268435456.f), -(1 << 30)), 1 << 30);
    const int q = qa + qb;
    const int carry = q >> kFracBits;  // floor(q / 2^28): the cell moves by carry
    int fi = (int)f + carry;
    u = fmaf(2.f, (float)carry, u);    // 1 - 2 (a - carry)
    if ((unsigned)fi >= (unsigned)dims) {
        fi %= dims;
        if (fi < 0)
            fi += dims;
    }
    return {fi, (uint32_t)q & (kFracOne - 1u), u, xlu};
}

// split_q28 where 1 <= |xh| < 2^22, xh = p * uh rounded as split_q28 rounds
// it, without the wrap into [0, dims): the same cell (before the wrap),
// fraction, u and xl.  In that range split_q28's near-origin step does not
// apply and |xl| < 2^22 * 2^-23, so xl * 2^28 needs no clamp.  The caller
// wraps the (rare) cells outside [0, dims).
constexpr float kFastSplitMax = 4194304.f;  // 2^22 cells

__device__ __forceinline__ AxisQ split_q28_unwrapped(float p, float xh, float uh, float ul)
{
    const float xe = fmaf(p, uh, -xh);
    const float xl = fmaf(p, ul, xe);
    const float f = floorf(xh);
    const float a = __fsub_rn(xh, f);
    float u = fmaf(-2.f, a, 1.f);
    const int q = __float2int_rn(a * 268435456.f) + __float2int_rn(xl * 268435456.f);
    const int carry = q >> kFracBits;
    u = fmaf(2.f, (float)carry, u);
    return {(int)f + carry, (uint32_t)q & (kFracOne - 1u), u, xl};
}

__device__ __forceinline__ int wrap_cell(int fi, int dims)
{
    if ((unsigned)fi >= (unsigned)dims) {
        fi %= dims;
        if (fi < 0)
            fi += dims;
    }
    return fi;
}

// The CIC weights of one particle in 2^-s mass units, shared by every deposit
// path so that they produce identical integer cell sums.  Factors per axis:
// 2^28 - q (lower cell) and q (upper), so f / 2^28 is the CIC factor; the
// particle's mass is mant * 2^(e - 150) (mant with its implicit bit) and
// dsh = emax - e for the pass's largest exponent emax, with s = 154 - emax.
//   pair (x, y):  P = rnd(fx fy / 2^26)                 <= 2^30
//   z with mass:  Z = rnd(rnd(fz mant / 2^23) / 2^dsh)  <= 2^29
//   corner:       W = rnd(P Z / 2^31)                   <= 2^28
// so W = prod(f / 2^28) * m * 2^s to within ~2 units.  rnd is to nearest: a
// truncation bias depends on the fraction, and on a lattice that follows the
// displacement field.  Each rnd(a b / 2^32) is one 32x32->64 multiply plus a
// 64-bit add; the operands are pre-scaled so the binary point sits at bit 32.
__device__ __forceinline__ uint32_t mul_rnd_hi(uint32_t a, uint32_t b)
{
    return (uint32_t)(((unsigned long long)a * b + 0x80000000ull) >> 32);
}

__device__ __forceinline__ uint32_t pair_w(uint32_t fx, uint32_t fy)
{
    return mul_rnd_hi(fx << 3, fy << 3);  // fx, fy <= 2^28: fx fy 2^6 / 2^32
}

__device__ __forceinline__ uint32_t z_mass(uint32_t fz, uint32_t mant, int dsh)
{
    const uint32_t z = mul_rnd_hi(fz << 3, mant << 6);  // fz mant 2^9 / 2^32
    if (dsh == 0)
        return z;
    if (dsh > 31)
        return 0u;
    return (uint32_t)(((unsigned long long)z + (1ull << (dsh - 1))) >> dsh);
}

__device__ __forceinline__ uint32_t corner_w(uint32_t p, uint32_t z)
{
    return mul_rnd_hi(p, z << 1);  // p z 2 / 2^32 = p z / 2^31
}

// prod_a (1 - 2 d_a) = prod_a (u_a - 2 xl_a) as a float pair: the product of
// the u's with two-product steps (relative error ~2^-47), then the first-,
// second- and third-order xl terms in FP32.  All orders are kept: xl holds
// p * (units - fl(units)), up to x * 2^-24, and dropping the second order left
// a coherent error of ~1e-4 in the single-mode last bin of a 128^3 lattice.
__device__ __forceinline__ f2sum corner_factor_q(const AxisQ &x, const AxisQ &y, const AxisQ &z)
{
    // (u_x + l_x)(u_y + l_y) with l = -2 xl: P exact to ~2^-47 relative plus
    // E = its rounding error + u_x l_y + l_x u_y + l_x l_y; then times
    // (u_z + l_z) the same way, so the first-, second- and third-order l
    // terms all enter E3 (each in FP32).
    const float lx = -2.f * x.xl, ly = -2.f * y.xl, lz = -2.f * z.xl;
    const float p = __fmul_rn(x.u, y.u);
    float e = fmaf(x.u, y.u, -p);
    e = fmaf(x.u, ly, e);
    e = fmaf(lx, y.u, e);
    e = fmaf(lx, ly, e);
    const float p3 = __fmul_rn(p, z.u);
    float e3 = fmaf(p, z.u, -p3);
    e3 = fmaf(p, lz, e3);
    e3 = fmaf(e, z.u, e3);
    e3 = fmaf(e, lz, e3);
    return {p3, e3};
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
