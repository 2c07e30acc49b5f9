// nb_common.cuh -- data layout and device helpers shared by the nonbonded kernels.
//
// Device layout (one handle, any number of replicas):
//   caller order : atoms in MOIL order, replica-major (coor(3,npt) of each replica back to back)
//   site order   : atoms regrouped for the pair kernels, rebuilt at every list build:
//                  [0, 3*nW)        water sites, molecule m -> sites 3m (O), 3m+1, 3m+2 (H, H)
//                  [3*nW, nsite)    non-water atoms
//                  waters and non-water atoms are each ordered by (replica, cell, unit id)
//   units        : one per water molecule (anchor = O) and one per non-water atom
//
// Fixed point: pair-kernel gradients are accumulated per lane in FP32 over short chunks
// and flushed to int64 at 2^32 units per kcal/mol/Å; integer addition makes the total
// independent of summation order, so forces are bit-identical run to run.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "erfcx_coef.h"

#define NB_KOFDIE 332.0716            // COMMON/CONVERT.BLOCK:13
#define NB_FIX_SCALE 4294967296.0     // 2^32
#define NB_FIX_SCALE_F 4294967296.0f
#define NB_FIX_INV (1.0 / 4294967296.0)
#define NB_PLANE_SCALE 1099511627776.0  // 2^40: PME plane accumulation
#define NB_MAX_FFT 128
#define NB_TWO_OVER_SQRTPI 1.1283791670955126
#define NB_EU 8                       // per-unit outputs: LJ prim, LJ img, Coul prim, Coul img, site pairs,
                                      // intramolecular water correction (mixed path), LJ virial prim, img
#define NB_EX 4                       // per-atom outputs: exclusion correction, 1-4 Coulomb, 1-4 LJ, 1-4 LJ virial
#define NB_EREP 24                    // per-replica results (energies, pair count, LJ virial terms)
#define NB_WTILE 128                  // waters per block (and per shared tile) of the tiled water list

// per-replica constants (read by every kernel)
struct RepDev {
    int atom0, natom;        // caller atoms
    int wat0, nwat;          // sorted water molecules [wat0, wat0+nwat)
    int oth0, noth;          // sorted non-water atoms (index into the non-water block)
    int cell0, nc[3];        // cell grid
    float L[3], invL[3];
    float Llo[3];            // Ld - (double)L: the box shift is applied as L + Llo so FP32
                             // image displacements carry no box-rounding bias
    double Ld[3], invLd[3];
    float rv2, re2, rmax2;   // LJ cutoff^2, Coulomb cutoff^2, max of both
    float rlist2;            // (rmax + skin)^2 : list radius between anchors of like units
    float rlistw2;           // (rmax + skin + 2*rwat)^2 : list radius anchor-to-anchor, mixed units
    float alpha, ex2c;       // alpha, alpha^2 * log2(e)
    float c2a;               // 2 alpha / sqrt(pi)
    double alphad;
    float ron2, swden;       // LJ switch (extension)
    float qq[3];             // water qO*qO, qO*qH, qH*qH times kofdie/eps (pot/watwat_ewald.f:70-79)
    float w12, w6;           // water O-O LJ A, B (pot/watwat_ewald.f:62-68)
    double qqd[3], w12d, w6d;
    float w12c, w6c;         // relative FP32 rounding of w12, w6: (w12d - w12) / w12, (w6d - w6) / w6
    double pme_qcorr;        // FP32 path: sum (q fc)^2 over the sum of the squared FP32 spread charges
    double epstmp;           // kofdie / eps
    int n1, n2, n3, n1h;     // PME grid, n1h = n1/2 + 1
    long long g0;            // first complex element of this replica's half-complex grid
    int zb0;                 // first z-bin of this replica
    int bsp0;                // bsp moduli: [bsp0, +n1) x, [+n1, +n2) y, [+n2, +n3) z
    float fc;                // sqrt(kofdie/eps)
    double fcd;
    float spread_scale;      // FP32 path: plane accumulation in int32 units of 1/spread_scale,
    float spread_inv;        // a power of two from nb_spread_exp
    float spread216;         // FP32 spread factor spread_scale / 216 (weights taken as 6 theta)
    double spread216_corr;   // (spread_scale / 216) / spread216
    double pme_fac;          // pi^2 / alpha^2
    double pivol;            // pi * volume
    float pme_fac2f, pivolf; // FP32 path: pi^2 / alpha^2 * log2(e), pi * volume
    float pme_gs[3];         // FP32 path: fc * n_d / L_d (PME gradient scale per unit charge)
    int arith, hvdw0, lj_switch, has_water;
    int wtiled;              // water-water list by tiled all-pairs (few cells per box)
    double e_self;
    double pivol_corr;       // FP32 path: (double)pivolf / pivol, applied to the FP64 energy sums
    float msq_c[3][2];       // FP32 path: invL_d^2 as hi + lo (accurate m^2 in the influence function)
    float fac2_lo;           // FP32 path: pme_fac2f's rounding remainder
    float invL_lo[3];        // FP32 path: invLd - (double)invL (PME fractional coordinates)
    // Water exclusion energies relative to a reference water (mixed path, wref != 0): every water
    // of the replica carries the charges of its last one, and the energy of a water's three
    // intramolecular pairs (O-H, O-H, H-H) is wcorr0 (FP64, exact erf at the squared reference
    // distances wt0) plus coef * (r^2 - wt0) * Q(r^2) in FP32, Q the quotient of the erf(x)/x
    // series in r^2 by (r^2 - wt0): a small difference, so FP32 rounding stays negligible
    int wref;
    int wsame;               // every water has the charges (qO, qH, qH) of the last one (host check)
    int wfirst;              // caller atom of the first water's O (the reference geometry), or -1
    float wt0[2];            // reference r^2 of the O-H and H-H pairs (FP32 values)
    float wcoef[2];          // -qq kofdie/eps alpha 2/sqrt(pi) of the O-H and H-H pairs
    float wq[2][8];          // quotient polynomial coefficients, ascending powers of r^2
    double wcorr0;           // exclusion energy of one reference water
};

// Exponent k of the int32 PME plane scale 2^k (FP32 path): one atom's largest stencil weight,
// q fc (2/3)^3, times 2^k stays below 2^25, so a grid point holds the sum of 64 such maximal
// contributions without overflow (the stencil weights of atoms around one grid point sum to
// about 1 on a 1 Å grid and about 2.3 on a 1.9 Å grid) at a resolution of 2^-25 of the
// largest contribution
__host__ __device__ inline int nb_spread_exp(double qfc_max)
{
    const double contrib = qfc_max * (8.0 / 27.0);
    int k = contrib > 0 ? (int)floor(log2(33554432.0 / contrib)) : 28;
    return k < 8 ? 8 : (k > 28 ? 28 : k);
}

// PME fractional grid coordinates of a site.  FP64 path: fr in [0, n] as a double.  FP32 path:
// fr as fixed point with 2^23 units per grid point (n <= 128, so below 2^30), kept in the bits
// of a float -- a single FP32 value near n would hold the fraction to only 2^-24 n.
__device__ __forceinline__ float pme_fr_pack(int i, float w)
{
    return __int_as_float((i << 23) + min(__float2int_rn(w * 8388608.f), 8388607));
}
__device__ __forceinline__ void pme_fr_split(float v, int &i, float &w)
{
    const int b = __float_as_int(v);
    i = b >> 23;
    w = __int2float_rn(b & 0x7fffff) * (1.f / 8388608.f);
}
__device__ __forceinline__ void pme_fr_split(double v, int &i, double &w)
{
    i = (int)v;
    w = v - (double)i;
}

// site flags
#define SF_CHARGED 1u        // |q| > 1e-6 (connect/chsort.f:17-24)
#define SF_WATER 2u
#define SF_HTINY 4u          // geometric rule: epsgm12 < 1e-3 (pot/nbond.f:115-126)

// a chunk of one replica's per-unit, per-atom or per-column energy partials (the energy
// reduction): kind 0 water units, 1 other units, 2 atoms, 3 PME column items; [begin, end)
struct EChunk { int rep, kind, begin, end; };
#define NB_FE_SEG 1024

// work descriptors for the PME plane / column kernels
struct PlaneWork { int rep, z; };
struct ColWork { int rep, kx, ky0, nky; };   // z columns at fixed kx for ky in [ky0, ky0 + nky)

// ---------------------------------------------------------------------------------
// precision traits

template <typename T> struct vec4;
template <> struct vec4<float> { typedef float4 type; };
template <> struct vec4<double> { typedef double4 type; };
template <typename T> struct cplx;
template <> struct cplx<float> { typedef float2 type; };
template <> struct cplx<double> { typedef double2 type; };

// single MUFU instructions, denormals flushed (arguments here are never denormal):
// rsqrt/rcp/ex2 .approx.ftz.f32 (relative error of order 2^-22)
__device__ __forceinline__ float nb_rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float nb_rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float nb_ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// L1 prefetch hint; callers pass addresses inside their own allocation
__device__ __forceinline__ void nb_prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

__device__ __forceinline__ float nb_rint(float x) { return rintf(x); }
__device__ __forceinline__ double nb_rint(double x) { return rint(x); }
__device__ __forceinline__ float nb_rsqrt(float x) { return nb_rsqrt_approx(x); }
__device__ __forceinline__ double nb_rsqrt(double x) { return rsqrt(x); }

template <typename T> __device__ __forceinline__ T rep_L(const RepDev &r, int k);
template <> __device__ __forceinline__ float rep_L<float>(const RepDev &r, int k) { return r.L[k]; }
template <> __device__ __forceinline__ double rep_L<double>(const RepDev &r, int k) { return r.Ld[k]; }
template <typename T> __device__ __forceinline__ T rep_invL(const RepDev &r, int k);
template <> __device__ __forceinline__ float rep_invL<float>(const RepDev &r, int k) { return r.invL[k]; }
template <> __device__ __forceinline__ double rep_invL<double>(const RepDev &r, int k) { return r.invLd[k]; }

// t - n*L for the image shift n, with the box length split in two FP32 parts (FP32) or
// exact (FP64)
__device__ __forceinline__ float nb_shift(const RepDev &R, int k, float t, float n)
{
    return fmaf(-n, R.Llo[k], fmaf(-n, R.L[k], t));
}
__device__ __forceinline__ double nb_shift(const RepDev &R, int k, double t, double n) { return t - n * R.Ld[k]; }

// erfc(x) and the derivative factor for the Ewald real-space term.
//   FP32: erfc(x) = exp(-x^2) * erfcx(x); erfcx from the fitted form in erfcx_coef.h,
//         exp(-x^2) = exp2(-x^2 log2 e).
//   FP64: libdevice erfc / exp.
// Returns erfc(x); *ex = exp(-x^2).
__device__ __forceinline__ float nb_erfc_ex(float x, float x2log2e, float *ex)
{
    const float C[ERFCX_NC] = ERFCX_COEFS;
    float xc = fminf(x, 4.5f);
    float t = nb_rcp_approx(fmaf(ERFCX_P, xc, 1.0f));
    float u = fmaf(ERFCX_A, t, ERFCX_B);
    float p = C[ERFCX_NC - 1];
#pragma unroll
    for (int k = ERFCX_NC - 2; k >= 0; --k) p = fmaf(p, u, C[k]);
    float e = nb_ex2_approx(-x2log2e);
    *ex = e;
    return e * (t * p);
}

__device__ __forceinline__ double nb_erfc_ex(double x, double /*unused*/, double *ex)
{
    *ex = exp(-x * x);
    return erfc(x);
}

// v * 2^32 rounded to nearest (ties away from zero) with integer operations only: a 64-bit
// conversion instruction runs on the narrow FP64 pipe.  |v| >= 2^31, Inf and NaN saturate
// to +-2^62.
__device__ __forceinline__ long long nb_f2fix(float v)
{
    const unsigned b = __float_as_uint(v);
    const int e = (int)((b >> 23) & 0xffu);
    const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - 118;    // v = m * 2^(e - 150), times 2^32
    long long r;
    if (sh > 38) r = 1LL << 62;
    else if (sh >= 0) r = m << sh;
    else if (sh > -26) r = (m + (1LL << (-sh - 1))) >> -sh;
    else r = 0;
    return (b >> 31) ? -r : r;
}

// x * 2^-32 as a double with integer operations only; exact for |x| < 2^53, truncated above
__device__ __forceinline__ double nb_fix2d(long long x)
{
    if (x == 0) return 0.0;
    const unsigned long long s = x < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long a = x < 0 ? 0ull - (unsigned long long)x : (unsigned long long)x;
    const int lz = __clzll((long long)a);
    const unsigned long long m = lz >= 11 ? a << (lz - 11) : a >> (11 - lz);
    const unsigned long long ex = (unsigned long long)(1023 + 31 - lz);
    return __longlong_as_double((long long)(s | (ex << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

// 64-bit fixed-point flush of an FP32 partial gradient (conversion instruction: cheaper
// than nb_f2fix where the FP64 pipe is otherwise idle)
__device__ __forceinline__ long long nb_fix(float v) { return __float2ll_rn(v * NB_FIX_SCALE_F); }
__device__ __forceinline__ long long nb_fix(double v) { return __double2ll_rn(v * NB_FIX_SCALE); }

// Owner of the water pair (a, b) in the half lists (indices relative to the replica's first
// water): the lower index when a + b is odd, the higher one when it is even.  Each water owns
// about half of its partners whatever its position in the sorted order.
__host__ __device__ __forceinline__ int nb_half_owner(int a, int b)
{
    return ((a ^ b) & 1) ? min(a, b) : max(a, b);
}

// Half-list water kernel: j-side gradients are summed per block in int32 at 2^(24 - log2 HB)
// units per kcal/mol/Å, so HB contributions of magnitude below NB_HALF_CAP cannot overflow;
// a larger contribution goes straight to the int64 site gradient
#define NB_HALF_CAP 127.0f

// bounded-status helpers
#define NB_DEV_ERR_OVERFLOW 1
#define NB_DEV_ERR_NAN 2
#define NB_DEV_ERR_BIGFORCE 4
#define NB_DEV_ERR_RWAT 8
