// adjoint.cu -- gradient of a P(k) loss with respect to particle positions and
// masses.  The reference computes no derivative; this is the exact adjoint of
// the forward path in deposit.cu / spectrum.cu:
//
//   P_b = S_b / (M^2 C_b),  S_b = sum_{m in b} c_m |F_m|^2 V_m,  F = r2c(rho)
//   dL/drho(x) = sum_m (2 g_b c_m V_m / (M^2 C_b)) Re(F_m e^{ikx}),  g_b = dL/dP_b
//
// evaluated as an unnormalised c2r of H_m = G_b * V_m * (c_m / mult_m) * F_m with
// G_b = 2 g_b / (M^2 C_b) and mult_m the c2r multiplicity of the mode (1 on the
// self-conjugate kz = 0 and, for even N, kz = N/2 planes, 2 elsewhere).  The
// position and mass gradients are then the CIC gather (transpose of the
// deposit) of dL/drho.  For N = 64..512 (powers of two) the mode gradient is
// applied inside the inverse x pass instead (xfft.cu, k_xfft<N, kXGrad>);
// k_mode_gradient here serves the other sizes.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace genpk {
namespace {

__device__ __forceinline__ int kval_adj(int i, int dims)
{
    return i <= dims / 2 ? i : i - dims;
}

struct ModeGradParams {
    int dims, hc, half;
    int nrbins;
    float bpu_half;
};

// One warp per (x, y) row of the half-complex spectrum: kx, ky, iw(kx) iw(ky)
// and kx^2 + ky^2 once per row (no 64-bit division per mode), lanes over kz,
// U modes per lane loaded before any is used.  Along a lane's kz the modulus
// only grows, so after one log-guided lookup its bin only steps up.
__global__ void __launch_bounds__(256)
    k_mode_gradient(ModeGradParams p, float2 *__restrict__ spec, const uint32_t *__restrict__ thr_g,
                    const float *__restrict__ iw, const float *__restrict__ gcoef)
{
    constexpr int U = 8;
    extern __shared__ uint32_t thr[];
    for (int i = threadIdx.x; i <= p.nrbins; i += blockDim.x)
        thr[i] = thr_g[i];
    __syncthreads();
    const bool even = (p.dims & 1) == 0;
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    const int nrows = p.dims * p.dims;
    for (int row = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); row < nrows;
         row += nwarps) {
        const int i = row / p.dims, j = row - i * p.dims;
        const int ki = kval_adj(i, p.dims), kj = kval_adj(j, p.dims);
        const uint32_t r2 = (uint32_t)(ki * ki + kj * kj);
        const float wij = __ldg(iw + i) * __ldg(iw + j);
        float2 *rp = spec + (size_t)row * (size_t)p.hc;
        int b = -1;
        for (int kz0 = 0; kz0 < p.hc; kz0 += 32 * U) {
            float2 f[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int kz = kz0 + lane + 32 * u;
                f[u] = kz < p.hc ? rp[kz] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int kz = kz0 + lane + 32 * u;
                if (kz >= p.hc)
                    break;
                const uint32_t kk2 = r2 + (uint32_t)(kz * kz);
                float2 h = make_float2(0.f, 0.f);
                if (kk2 != 0) {
                    if (b < 0) {
                        b = (int)(p.bpu_half * __logf((float)kk2));
                        b = max(0, min(p.nrbins - 1, b));
                        while (b > 0 && kk2 < thr[b])
                            b--;
                    }
                    while (b + 1 < p.nrbins && kk2 >= thr[b + 1])
                        b++;
                    const float pz = wij * __ldg(iw + kz);
                    const float p2 = pz * pz;
                    const bool edge = (kz == 0 || kz == p.half);               // reference weight 1
                    const bool selfconj = (kz == 0) || (even && kz == p.half);  // c2r counts once
                    const float cm = edge ? 1.f : 2.f;
                    const float mult = selfconj ? 1.f : 2.f;
                    const float sc = __ldg(gcoef + b) * (p2 * p2) * (cm / mult);
                    h = make_float2(sc * f[u].x, sc * f[u].y);
                }
                rp[kz] = h;
            }
        }
    }
}

// The mode gradient on a kz-major spectrum S[kz][x][y] (the N = 1024
// transform), in place: one warp per (kz, x) row, lanes over y; the same
// H = G_b V_m (c_m / mult_m) F_m as k_mode_gradient, p = (iw_x iw_y) iw_kz.
__global__ void __launch_bounds__(256)
    k_mode_gradient_kz(ModeGradParams p, float2 *__restrict__ spec,
                       const uint32_t *__restrict__ thr_g, const float *__restrict__ iw,
                       const float *__restrict__ gcoef)
{
    extern __shared__ uint32_t thr[];
    for (int i = threadIdx.x; i <= p.nrbins; i += blockDim.x)
        thr[i] = thr_g[i];
    __syncthreads();
    const bool even = (p.dims & 1) == 0;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nrows = (int64_t)p.hc * p.dims;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrows;
         row += nwarps) {
        const int kz = (int)(row / p.dims), x = (int)(row - (int64_t)kz * p.dims);
        const int kx = kval_adj(x, p.dims);
        const uint32_t r2 = (uint32_t)(kx * kx + kz * kz);
        const float iwx = __ldg(iw + x), iwz = __ldg(iw + kz);
        const bool edge = (kz == 0 || kz == p.half);
        const bool selfconj = (kz == 0) || (even && kz == p.half);
        const float cm = edge ? 1.f : 2.f, mult = selfconj ? 1.f : 2.f;
        float2 *rp = spec + (size_t)row * (size_t)p.dims;
        for (int y = lane; y < p.dims; y += 32) {
            const int ky = kval_adj(y, p.dims);
            const uint32_t kk2 = r2 + (uint32_t)(ky * ky);
            float2 h = make_float2(0.f, 0.f);
            if (kk2 != 0) {
                int b = (int)(p.bpu_half * __logf((float)kk2));
                b = max(0, min(p.nrbins - 1, b));
                while (b + 1 < p.nrbins && kk2 >= thr[b + 1])
                    b++;
                while (b > 0 && kk2 < thr[b])
                    b--;
                const float pz = (iwx * __ldg(iw + y)) * iwz;
                const float p2 = pz * pz;
                const float sc = __ldg(gcoef + b) * (p2 * p2) * (cm / mult);
                const float2 f = rp[y];
                h = make_float2(sc * f.x, sc * f.y);
            }
            rp[y] = h;
        }
    }
}

struct GatherParams {
    int dims;
    int64_t plane;
    int row;
    float uh, ul;
    float units;
    float mass;
    float dl_dm;
    int64_t n;
};

// The trilinear value and the three derivatives of dL/drho at one particle.
struct GatherOut {
    float gx, gy, gz, val;
};

__device__ __forceinline__ GatherOut gather_one(const GatherParams &p, const float *__restrict__ grid,
                                                float x, float y, float z, float m)
{
    int c[3];
    float d[3];
    split_cell(x, p.uh, p.ul, p.dims, c[0], d[0]);
    split_cell(y, p.uh, p.ul, p.dims, c[1], d[1]);
    split_cell(z, p.uh, p.ul, p.dims, c[2], d[2]);
    int h[3];
#pragma unroll
    for (int a = 0; a < 3; a++)
        h[a] = c[a] + 1 == p.dims ? 0 : c[a] + 1;
    float g[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
        g[k] = __ldg(grid + cell_index(p.plane, p.row, (k & 1) ? h[0] : c[0], (k & 2) ? h[1] : c[1],
                                       (k & 4) ? h[2] : c[2]));
    const float t0 = 1.f - d[0], t1 = 1.f - d[1];
    // Interpolate along z first, then y, then x; derivatives from the same tree.
    const float g00 = fmaf(d[2], g[4] - g[0], g[0]);  // (x0,y0)
    const float g10 = fmaf(d[2], g[5] - g[1], g[1]);  // (x1,y0)
    const float g01 = fmaf(d[2], g[6] - g[2], g[2]);  // (x0,y1)
    const float g11 = fmaf(d[2], g[7] - g[3], g[3]);  // (x1,y1)
    const float gx0 = fmaf(d[1], g01 - g00, g00);
    const float gx1 = fmaf(d[1], g11 - g10, g10);
    const float val = fmaf(d[0], gx1 - gx0, gx0);
    const float dgx = gx1 - gx0;
    const float gy0 = fmaf(d[0], g10 - g00, g00);
    const float gy1 = fmaf(d[0], g11 - g01, g01);
    const float dgy = gy1 - gy0;
    // d/dz: bilinear in (x, y) of the z-differences.
    const float e00 = g[4] - g[0], e10 = g[5] - g[1], e01 = g[6] - g[2], e11 = g[7] - g[3];
    const float dgz = t0 * (t1 * e00 + d[1] * e01) + d[0] * (t1 * e10 + d[1] * e11);
    const float s = m * p.units;
    return {s * dgx, s * dgy, s * dgz, val};
}

// One particle per thread, grid-stride.  (Tiles of 1024 particles staged
// through shared memory with 16-byte loads and stores, four particles per
// thread, ran slower: 1.20 ms against 0.93 at 512^3, with fewer warps resident
// to cover the grid loads' latency.)  Non-finite positions get zero gradients.
template <bool VARMASS>
__global__ void __launch_bounds__(256)
    k_gather(GatherParams p, const float *__restrict__ grid, const float *__restrict__ pos,
             const float *__restrict__ masses, float *__restrict__ gpos, float *__restrict__ gmass)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        const float m = VARMASS ? masses[i] : p.mass;
        if (!finite3(x, y, z)) {
            gpos[3 * i] = gpos[3 * i + 1] = gpos[3 * i + 2] = 0.f;
            if (VARMASS)
                gmass[i] = 0.f;
            continue;
        }
        const GatherOut o = gather_one(p, grid, x, y, z, m);
        gpos[3 * i] = o.gx;
        gpos[3 * i + 1] = o.gy;
        gpos[3 * i + 2] = o.gz;
        if (VARMASS)
            gmass[i] = o.val + p.dl_dm;
    }
}

// Four consecutive particles per thread: three 16-byte loads of positions
// (and one of masses), the 32 grid loads of the four particles issued
// together, three 16-byte stores of gradients.  The one-particle kernel's
// thread waits out a position load and then the grid loads for every
// particle; here each wait covers four.  Needs pos, gpos (and masses, gmass)
// on 16-byte boundaries; the last n % 4 particles go one per thread.
__device__ __forceinline__ GatherOut gather_or_zero(const GatherParams &p, const float *__restrict__ grid,
                                                    float x, float y, float z, float m)
{
    if (!finite3(x, y, z))
        return {0.f, 0.f, 0.f, -p.dl_dm};
    return gather_one(p, grid, x, y, z, m);
}

template <bool VARMASS>
__global__ void __launch_bounds__(256)
    k_gather4(GatherParams p, const float *__restrict__ grid, const float *__restrict__ pos,
              const float *__restrict__ masses, float *__restrict__ gpos, float *__restrict__ gmass)
{
    const int64_t groups = p.n >> 2;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t q = tid; q < groups; q += (int64_t)gridDim.x * blockDim.x) {
        const float4 *s = reinterpret_cast<const float4 *>(pos) + 3 * q;
        const float4 a = __ldg(s), b = __ldg(s + 1), c = __ldg(s + 2);
        float4 m = make_float4(p.mass, p.mass, p.mass, p.mass);
        if (VARMASS)
            m = __ldg(reinterpret_cast<const float4 *>(masses) + q);
        const GatherOut o0 = gather_or_zero(p, grid, a.x, a.y, a.z, m.x);
        const GatherOut o1 = gather_or_zero(p, grid, a.w, b.x, b.y, m.y);
        const GatherOut o2 = gather_or_zero(p, grid, b.z, b.w, c.x, m.z);
        const GatherOut o3 = gather_or_zero(p, grid, c.y, c.z, c.w, m.w);
        float4 *d = reinterpret_cast<float4 *>(gpos) + 3 * q;
        d[0] = make_float4(o0.gx, o0.gy, o0.gz, o1.gx);
        d[1] = make_float4(o1.gy, o1.gz, o2.gx, o2.gy);
        d[2] = make_float4(o2.gz, o3.gx, o3.gy, o3.gz);
        if (VARMASS)
            reinterpret_cast<float4 *>(gmass)[q] =
                make_float4(o0.val + p.dl_dm, o1.val + p.dl_dm, o2.val + p.dl_dm, o3.val + p.dl_dm);
    }
    const int64_t i = 4 * groups + tid;  // the last n % 4 particles
    if (i < p.n) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        const GatherOut o = gather_or_zero(p, grid, x, y, z, VARMASS ? masses[i] : p.mass);
        gpos[3 * i] = o.gx;
        gpos[3 * i + 1] = o.gy;
        gpos[3 * i + 2] = o.gz;
        if (VARMASS)
            gmass[i] = o.val + p.dl_dm;
    }
}

bool aligned16(const void *ptr)
{
    return ((uintptr_t)ptr & 15) == 0;
}

}  // namespace

cudaError_t adjoint_mode_gradient_kz(const GridGeom &g, const BinTables &t, const BinDevice &d,
                                     float2 *spec, const float *gcoef_dev, int num_sms,
                                     cudaStream_t stream, int64_t *launches)
{
    ModeGradParams p;
    p.dims = g.dims;
    p.hc = g.hc;
    p.half = g.half;
    p.nrbins = t.nrbins;
    p.bpu_half = (float)(0.5 * t.binsperunit);
    const size_t smem = sizeof(uint32_t) * (size_t)(t.nrbins + 1);
    cudaError_t err;
    if ((err = ensure_dynamic_smem(k_mode_gradient_kz, smem)) != cudaSuccess)
        return err;
    k_mode_gradient_kz<<<num_sms * 8, 256, smem, stream>>>(p, spec, d.thr, d.iw, gcoef_dev);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t adjoint_mode_gradient_coef(const GridGeom &g, const BinTables &t, const BinDevice &d,
                                       float2 *spec, const float *gcoef_dev, cudaStream_t stream,
                                       int64_t *launches)
{
    ModeGradParams p;
    p.dims = g.dims;
    p.hc = g.hc;
    p.half = g.half;
    p.nrbins = t.nrbins;
    p.bpu_half = (float)(0.5 * t.binsperunit);
    // one warp per row of kz modes; 4 CTAs of 8 warps per SM (46 registers)
    const int blocks = (int)std::min<int64_t>(((int64_t)g.dims * g.dims + 7) / 8, 152 * 4);
    k_mode_gradient<<<blocks, 256, sizeof(uint32_t) * (t.nrbins + 1), stream>>>(p, spec, d.thr,
                                                                              d.iw, gcoef_dev);
    (*launches)++;
    return cudaGetLastError();
}

cudaError_t adjoint_gather(const GridGeom &g, float units_hi, float units_lo, const float *grid,
                           const float *pos, const float *masses, float mass, int64_t n,
                           float *grad_pos, float *grad_mass, float dl_dmass_norm,
                           cudaStream_t stream, int64_t *launches)
{
    if (n <= 0)
        return cudaSuccess;
    GatherParams p;
    p.dims = g.dims;
    p.plane = g.plane;
    p.row = g.row;
    p.uh = units_hi;
    p.ul = units_lo;
    p.units = units_hi + units_lo;
    p.mass = mass;
    p.dl_dm = dl_dmass_norm;
    p.n = n;
    // Four CTAs per resident slot (8 per SM at 32-36 registers).  Sizing the
    // grid to the resident CTAs, so that the stride sweeps the particles in
    // order, cut the DRAM reads at 512^3 from 2.85 to 2.56 GB (2.15 GB of
    // positions and grid) but took 1.00 ms against 0.92.
    const bool vec = aligned16(pos) && aligned16(grad_pos) &&
                     (!masses || (aligned16(masses) && aligned16(grad_mass)));
    if (vec) {
        const int blocks4 = (int)std::min<int64_t>(std::max<int64_t>((n / 4 + 255) / 256, 1), 152 * 32);
        if (masses)
            k_gather4<true><<<blocks4, 256, 0, stream>>>(p, grid, pos, masses, grad_pos, grad_mass);
        else
            k_gather4<false><<<blocks4, 256, 0, stream>>>(p, grid, pos, masses, grad_pos, grad_mass);
        (*launches)++;
        return cudaGetLastError();
    }
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 32);
    if (masses)
        k_gather<true><<<blocks, 256, 0, stream>>>(p, grid, pos, masses, grad_pos, grad_mass);
    else
        k_gather<false><<<blocks, 256, 0, stream>>>(p, grid, pos, masses, grad_pos, grad_mass);
    (*launches)++;
    return cudaGetLastError();
}

}  // namespace genpk
