// The modular solver on the GPU: SerialSolver<ReflectingWalls, Recon, Riemann, SSPRK3,
// Bathymetry> (include/backend/serial/serial_solver.hpp:105-524) with every
// reconstruction (PiecewiseConst, MUSCL) and Riemann solver (HLL, Rusanov, ROE) the
// reference composes, with bathymetry (FluxAssemblyBathy, FiniteVolumeBathy, positivity)
// or without (FluxAssembly, FiniteVolume).
//
// One fused kernel per RK stage, as for the optimised solver: a block stages its tile
// of the source state (plus a 2-cell halo, walls by mirrored indices) in shared memory,
// computes every x- and y-interface flux its cells need into shared memory, then the
// finite-volume update, the SSP-RK3 combine and the positivity floor, and writes the
// tile's interior.  No flux or rhs array exists in HBM.
//
// The arithmetic is the reference's own, operation by operation, including the
// association of its CellState and std::array expressions, so results are bitwise equal
// to SerialSolver: the file is compiled with --fmad=false, and its divisions and square
// roots are correctly rounded (on the integer pipes, swe_soft_f64.cuh).  std::min / std::max are written as their definitions
// ((b < a) ? b : a, (a < b) ? b : a), which fixes their NaN and signed-zero behaviour.
#include <cuda_runtime.h>

#include <algorithm>

#include "swe_common.cuh"
#include "swe_launch.h"
#include "swe_soft_f64.cuh"

namespace swe {
namespace mod {

// tile: 8 x-rows by 32 y-columns; 288 threads, so that the tile's 552 interfaces are at
// most two per thread (with 256, a few threads took four and the rest waited at the barrier)
constexpr int TI = 8, TJ = 32, NT = (TI + 1) * TJ;
constexpr int RI = TI + 4, RJ = TJ + 4;        // staged rows / columns (2-cell halo)
constexpr double EPS = 1.0e-8;                 // constants::eps (include/constants.hpp:5)
constexpr int64_t EPS_BITS = 0x3E45798EE2308C3ALL;  // bits of 1.0e-8
constexpr double H_FLOOR = 1.0e-8;             // serial_solver.hpp:454

struct CS {
    double h, hu, hv;
};  // CellState (include/core/cell_state.hpp:6-35)

// A CellState with its u() and v() (cell_state.hpp:18-25), computed once: the reference
// recomputes them on every call, with the same operands, so the values are the same.
struct CSV {
    double h, hu, hv, u, v;
};

// Comparisons, min / max, |x|, 0.5 x and minmod on the bit patterns (swe_f64_exact.cuh):
// the IEEE decisions and values, NaN included, off the FP64 pipe, which otherwise spends
// about a third of its issue slots on them here.
__device__ __forceinline__ double dmin(double a, double b) { return x64::dmin(a, b); }  // std::min
__device__ __forceinline__ double dmax(double a, double b) { return x64::dmax(a, b); }  // std::max

// IEEE division and square root, correctly rounded on the integer pipes
// (swe_soft_f64.cuh): the same results as the FP64 unit's, off the FP64 pipe.
__device__ __forceinline__ double ddiv(double a, double b) { return sf::div_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return sf::sqrt_rn(a); }

__device__ __forceinline__ CSV with_velocity(const CS &s) {
    CSV r{s.h, s.hu, s.hv, 0.0, 0.0};
    if (x64::gt_pos_const(s.h, EPS_BITS)) sf::div2_rn(s.hu, s.hv, s.h, r.u, r.v);  // h > eps
    return r;
}

// RiemannSolver::F / G (riemann/riemann.hpp:10-19); half_g = 0.5 * g (exact).
__device__ __forceinline__ CS phys_flux(int DIR, double half_g, const CSV &U) {
    if (DIR == 0) return {U.hu, U.u * U.u * U.h + half_g * U.h * U.h, U.hu * U.v};
    return {U.hv, U.hu * U.v, U.h * U.v * U.v + half_g * U.h * U.h};
}

// HLL (riemann/HLL.hpp:10-45).  Sets *fail where the reference throws "HLL could not
// provide dissipation speed." (NaN speeds).
__device__ __forceinline__ CS hll(int DIR, double g, double half_g, const CSV &A, const CSV &B, bool *fail) {
    const double uA = DIR == 0 ? A.u : A.v, uB = DIR == 0 ? B.u : B.v;
    const double cA = dsqrt(g * A.h), cB = dsqrt(g * B.h);
    const double sR = dmax(uA + cA, uB + cB);
    const double sL = dmin(uA - cA, uB - cB);
    if (x64::le(0.0, sL)) return phys_flux(DIR, half_g, A);
    if (x64::lt(sL, 0.0) && x64::lt(0.0, sR)) {
        const CS FA = phys_flux(DIR, half_g, A), FB = phys_flux(DIR, half_g, B);
        const double ss = sL * sR, d = sR - sL;
        CS r;
        sf::div2_rn(sR * FA.h - sL * FB.h + ss * (B.h - A.h),
                    sR * FA.hu - sL * FB.hu + ss * (B.hu - A.hu), d, r.h, r.hu);
        r.hv = ddiv(sR * FA.hv - sL * FB.hv + ss * (B.hv - A.hv), d);
        return r;
    }
    if (x64::le(sR, 0.0)) return phys_flux(DIR, half_g, B);
    *fail = true;
    return {0.0, 0.0, 0.0};
}

// Rusanov (riemann/rusanov.hpp:12-30)
__device__ __forceinline__ CS rusanov(int DIR, double g, double half_g, const CSV &A, const CSV &B) {
    const double uA = DIR == 0 ? A.u : A.v, uB = DIR == 0 ? B.u : B.v;
    const double hB = dmax(B.h, 0.0), hA = dmax(A.h, 0.0);
    const double a = dmax(x64::fabs_(uA) + dsqrt(g * hA), x64::fabs_(uB) + dsqrt(g * hB));
    const CS FA = phys_flux(DIR, half_g, A), FB = phys_flux(DIR, half_g, B);
    const double ha = x64::halve(a);  // 0.5 * a
    return {x64::halve(FA.h + FB.h) - ha * (B.h - A.h),
            x64::halve(FA.hu + FB.hu) - ha * (B.hu - A.hu),
            x64::halve(FA.hv + FB.hv) - ha * (B.hv - A.hv)};
}

// ROE (riemann/ROE.hpp:10-63), compute_roe_avg (:66-69) for u and v over the one
// denominator sqrt(h1) + sqrt(h2).  The eigenvectors' 0 and 1 entries are multiplied as
// written: 0 * x keeps the sign of x and its NaN, as the reference's std::array product.
__device__ __forceinline__ CS roe(int DIR, double g, double half_g, const CSV &A, const CSV &B) {
    const double h = x64::halve(A.h + B.h);  // (A.h + B.h) / 2.0
    const double c = dsqrt(g * h);
    const double sA = dsqrt(A.h), sB = dsqrt(B.h);
    double u_roe, v_roe;
    sf::div2_rn((sA * A.u) + (sB * B.u), (sA * A.v) + (sB * B.v), sA + sB, u_roe, v_roe);
    const double vn = DIR == 0 ? u_roe : v_roe, vt = DIR == 0 ? v_roe : u_roe;
    const double l1 = vn - c, l2 = vn, l3 = vn + c;
    const double dh = B.h - A.h, dhu = B.hu - A.hu, dhv = B.hv - A.hv;
    const double dqn = DIR == 0 ? dhu : dhv, dqt = DIR == 0 ? dhv : dhu;
    const double q = ddiv(dqn - vn * dh, c);
    const double alpha1 = x64::halve(dh - q);
    const double alpha3 = x64::halve(dh + q);
    const double alpha2 = dqt - vt * dh;
    const double w1 = x64::fabs_(l1) * alpha1, w2 = x64::fabs_(l2) * alpha2,
                 w3 = x64::fabs_(l3) * alpha3;
    // r1 = {1, l1, v_roe}, r2 = {0, 0, 1}, r3 = {1, l3, v_roe} in x;
    // r1 = {1, u_roe, l1}, r2 = {0, 1, 0}, r3 = {1, u_roe, l3} in y.
    const double r1[3] = {1.0, DIR == 0 ? l1 : u_roe, DIR == 0 ? v_roe : l1};
    const double r2[3] = {0.0, DIR == 0 ? 0.0 : 1.0, DIR == 0 ? 1.0 : 0.0};
    const double r3[3] = {1.0, DIR == 0 ? l3 : u_roe, DIR == 0 ? v_roe : l3};
    double sum[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) sum[k] = x64::halve((r1[k] * w1 + r2[k] * w2) + r3[k] * w3);
    const CS FA = phys_flux(DIR, half_g, A), FB = phys_flux(DIR, half_g, B);
    return {x64::halve(FA.h + FB.h) - sum[0], x64::halve(FA.hu + FB.hu) - sum[1],
            x64::halve(FA.hv + FB.hv) - sum[2]};
}

template <int RIEMANN>
__device__ __forceinline__ CS riemann(int DIR, double g, double half_g, const CS &A0,
                                      const CS &B0, bool *fail) {
    const CSV A = with_velocity(A0), B = with_velocity(B0);
    if (RIEMANN == 0) return hll(DIR, g, half_g, A, B, fail);
    if (RIEMANN == 1) return rusanov(DIR, g, half_g, A, B);
    return roe(DIR, g, half_g, A, B);
}

// minmod_scalar (reconstruction/muscl.hpp:7-10), the same expression as the optimised
// solver's minmod (HPC_kernels.hpp:41-44), so x64::minmod computes it
__device__ __forceinline__ double minmod_scalar(double a, double b) { return x64::minmod(a, b); }

struct Tile {
    double w[3][RI][RJ];  // eta (or h), hu, hv of the staged cells
    double b[RI][RJ];     // B of the staged cells (bathymetry only)
    // x-interfaces a = 0..TI between staged rows a+1 and a+2: h, hu of F^-, hu of F^+,
    // hv.  y-interfaces b = 0..TJ between staged columns b+1 and b+2: h, hu, hv of G^-,
    // hv of G^+.  (Without bathymetry F^- = F^+.)
    double fx[4][TI + 1][TJ];
    double fy[4][TI][TJ + 1];
};

__device__ __forceinline__ CS cell(const Tile &t, int r, int c) {
    return {t.w[0][r][c], t.w[1][r][c], t.w[2][r][c]};
}

// U_L / U_B and U_R / U_T of the interface between staged cells (r, c) and
// (r + DI, c + DJ): PiecewiseConst (piecewise_const.hpp:11-30) or MUSCL (muscl.hpp:14-66).
template <int RECON>
__device__ __forceinline__ void reconstruct(const Tile &t, int r, int c, int DI, int DJ, CS *A,
                                            CS *B) {
    const CS c0 = cell(t, r, c), c1 = cell(t, r + DI, c + DJ);
    if (RECON == 0) {
        *A = c0;
        *B = c1;
        return;
    }
    const CS cm = cell(t, r - DI, c - DJ), c2 = cell(t, r + 2 * DI, c + 2 * DJ);
    const CS s0 = {minmod_scalar(c0.h - cm.h, c1.h - c0.h), minmod_scalar(c0.hu - cm.hu, c1.hu - c0.hu),
                   minmod_scalar(c0.hv - cm.hv, c1.hv - c0.hv)};
    const CS s1 = {minmod_scalar(c1.h - c0.h, c2.h - c1.h), minmod_scalar(c1.hu - c0.hu, c2.hu - c1.hu),
                   minmod_scalar(c1.hv - c0.hv, c2.hv - c1.hv)};
    *A = {c0.h + x64::halve(s0.h), c0.hu + x64::halve(s0.hu), c0.hv + x64::halve(s0.hv)};
    *B = {c1.h - x64::halve(s1.h), c1.hu - x64::halve(s1.hu), c1.hv - x64::halve(s1.hv)};
}

// One interface: FluxAssemblyBathy (flux_assembly_bathy.hpp:18-192) or FluxAssembly
// (flux_assembly.hpp:11-45).  out: h, hu / hv of F^-, the same of F^+, the other momentum.
template <int RECON, int RIEMANN, bool BATHY>
__device__ __forceinline__ void interface_flux(int DIR, const Tile &t, int r, int c, double g,
                                               double half_g, double out[4], bool *fail) {
    const int DI = DIR == 0 ? 1 : 0, DJ = DIR == 0 ? 0 : 1;
    CS A, B;
    reconstruct<RECON>(t, r, c, DI, DJ, &A, &B);
    if (!BATHY) {
        const CS F = riemann<RIEMANN>(DIR, g, half_g, A, B, fail);
        const double qn = DIR == 0 ? F.hu : F.hv, qt = DIR == 0 ? F.hv : F.hu;
        out[0] = F.h;
        out[1] = qn;
        out[2] = qn;
        out[3] = qt;
        return;
    }
    const double eta_m = A.h, eta_p = B.h;
    const double b_m = t.b[r][c], b_p = t.b[r + DI][c + DJ];
    const double b_star = dmax(b_m, b_p);
    // positive_height = std::max(0.0, h), i.e. h > 0 ? h : 0.0
    const double h_m = x64::positive_part(eta_m - b_m), h_p = x64::positive_part(eta_p - b_p);
    // safe_velocity (flux_assembly_bathy.hpp:180-185)
    double u_m = 0.0, v_m = 0.0, u_p = 0.0, v_p = 0.0;
    if (!x64::lt(h_m, EPS)) sf::div2_rn(A.hu, A.hv, h_m, u_m, v_m);
    if (!x64::lt(h_p, EPS)) sf::div2_rn(B.hu, B.hv, h_p, u_p, v_p);
    const double hs_m = x64::positive_part(eta_m - b_star), hs_p = x64::positive_part(eta_p - b_star);
    const CS Um = {hs_m, hs_m * u_m, hs_m * v_m}, Up = {hs_p, hs_p * u_p, hs_p * v_p};
    const CS F = riemann<RIEMANN>(DIR, g, half_g, Um, Up, fail);
    const double corr_m = half_g * (h_m * h_m - hs_m * hs_m);
    const double corr_p = half_g * (h_p * h_p - hs_p * hs_p);
    const double qn = DIR == 0 ? F.hu : F.hv, qt = DIR == 0 ? F.hv : F.hu;
    out[0] = F.h;
    out[1] = qn + corr_m;
    out[2] = qn + corr_p;
    out[3] = qt;
}

struct ModParams {
    const double *hs, *hus, *hvs;  // stage source
    const double *hn, *hun, *hvn;  // U^n
    const double *B;
    double *ho, *huo, *hvo;
    int Nx, Ny;
    long long P;
    double g, half_g;
    double nidx, idy;  // -1.0 / dx and 1.0 / dy (finite_volume_bathy.hpp:17-27)
    int kx, ky;        // log2 of 1.0 / dx and 1.0 / dy when powers of two, else 127
    double dt, c2, c3; // dt, dt / 4.0, 2.0 * dt / 3.0 (ssp_rk3.hpp:12-37)
    int stage;
    int *flags;
};


// The RK combination's products: correctly rounded on the integer pipes when
// SWE_MOD_SOFT_CU is set (the same results; it moves work off the FP64 pipe).
#ifndef SWE_MOD_SOFT_CU
#define SWE_MOD_SOFT_CU 0
#endif
__device__ __forceinline__ double cu(double a, double b) {
#if SWE_MOD_SOFT_CU
    return sf::mul_rn(a, b);
#else
    return a * b;
#endif
}

// Reflecting walls by mirrored index (reflecting_walls.hpp:9-86): a ghost reads its
// mirror cell, with the normal momentum negated.
__device__ __forceinline__ int mirror(int i, int N, bool *flip) {
    if (i < 0) {
        *flip = true;
        return -1 - i;
    }
    if (i >= N) {
        *flip = true;
        return 2 * N - 1 - i;
    }
    *flip = false;
    return i;
}

// Resident CTAs per SM the register budget is sized for: four (56 registers, no spills)
// run 1-8% faster than the unbounded 70 registers and three CTAs.
#ifndef SWE_MOD_MIN_BLOCKS
#define SWE_MOD_MIN_BLOCKS 4
#endif

// Tiles per CTA: a CTA walks a strip of tiles along x and carries each tile's last
// x-interface row into the next, so that one x-interface row per strip is computed twice
// instead of one per tile.  The length is chosen per grid as for the fused kernel: six
// tiles while that leaves at least 16 waves of resident CTAs, else lone tiles
// (SWE_MOD_STRIP > 0 fixes it).
#ifndef SWE_MOD_STRIP
#define SWE_MOD_STRIP 0
#endif

template <int RECON, int RIEMANN, bool BATHY>
__global__ void __launch_bounds__(NT, SWE_MOD_MIN_BLOCKS) k_modular_stage(const ModParams p,
                                                                          int strip) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Tile &t = *reinterpret_cast<Tile *>(smem_raw);
    const int tid = threadIdx.x;
    const int tr0 = blockIdx.y * strip, j0 = blockIdx.x * TJ;
    const int n_tiles = min(strip, (p.Nx + TI - 1) / TI - tr0);
    bool fail = false, bad = false;
#pragma unroll 1
    for (int kt = 0; kt < n_tiles; ++kt) {
        const int i0 = (tr0 + kt) * TI;  // interior coordinates
        // Stage the tile and its halo.  Rows beyond the ghost layer (a ragged last tile)
        // are never read by a needed interface; they are zero-filled.
        for (int e = tid; e < RI * RJ; e += NT) {
            const int r = e / RJ, c = e - r * RJ;
            const int i = i0 + r - 2, j = j0 + c - 2;
            double h = 0.0, hu = 0.0, hv = 0.0, b = 0.0;
            if (i >= -2 && i < p.Nx + 2 && j >= -2 && j < p.Ny + 2) {
                bool fx, fy;
                const int mi = mirror(i, p.Nx, &fx), mj = mirror(j, p.Ny, &fy);
                const long long k = (long long)(mi + NG) * p.P + (mj + NG);
                h = p.hs[k];
                hu = fx ? -p.hus[k] : p.hus[k];
                hv = fy ? -p.hvs[k] : p.hvs[k];
                if (BATHY) {
                    b = p.B[k];
                    h = h + b;  // W.h() += B (flux_assembly_bathy.hpp:26-27)
                }
            }
            t.w[0][r][c] = h;
            t.w[1][r][c] = hu;
            t.w[2][r][c] = hv;
            if (BATHY) t.b[r][c] = b;
        }
        __syncthreads();  // staged; the previous tile's carried row is in place
        // One interface per thread and direction: the x-interface between staged rows a+1
        // and a+2 (interior rows i0+a-1 and i0+a), then, for the first TI * (TJ + 1)
        // threads, the y-interface between staged columns b+1 and b+2.  Both directions
        // run through one copy of the interface code (a loop, not unrolled): two inlined
        // copies of it stalled the kernel on instruction fetch.  After the first tile of
        // the strip, x-interface row 0 is the previous tile's row TI.
#pragma unroll 1
        for (int dir = 0; dir < 2; ++dir) {
            int r, c, q0, q1;  // staged cell of the interface's minus side; shared slots
            bool valid;
            if (dir == 0) {
                q0 = tid / TJ;
                q1 = tid - q0 * TJ;
                valid = (kt == 0 || q0 > 0) && i0 + q0 - 1 <= p.Nx - 1 && j0 + q1 < p.Ny;
                r = q0 + 1;
                c = q1 + 2;
            } else {
                q0 = tid / (TJ + 1);
                q1 = tid - q0 * (TJ + 1);
                valid = tid < TI * (TJ + 1) && i0 + q0 < p.Nx && j0 + q1 - 1 <= p.Ny - 1;
                r = q0 + 2;
                c = q1 + 1;
            }
            if (!valid) continue;
            double f[4];
            interface_flux<RECON, RIEMANN, BATHY>(dir, t, r, c, p.g, p.half_g, f, &fail);
            if (dir == 0) {
#pragma unroll
                for (int q = 0; q < 4; ++q) t.fx[q][q0][q1] = f[q];
            } else {
                t.fy[0][q0][q1] = f[0];
                t.fy[1][q0][q1] = f[3];  // hu
                t.fy[2][q0][q1] = f[1];  // hv of G^-
                t.fy[3][q0][q1] = f[2];  // hv of G^+
            }
        }
        __syncthreads();
        const int r = tid / TJ, c = tid - (tid / TJ) * TJ;
        const int i = i0 + r, j = j0 + c;
        if (r < TI && i < p.Nx && j < p.Ny) {
            // FiniteVolumeBathy / FiniteVolume::apply_spatial_operator: F^-(i) - F^+(i-1)
            // products by -1/dx and 1/dy: exact exponent shifts when they are powers of two
            auto mx = [&](double a) {
                return p.kx != 127 ? x64::neg(x64::scale2(a, p.kx, x64::neg(p.nidx))) : p.nidx * a;
            };
            auto my = [&](double a) { return p.ky != 127 ? x64::scale2(a, p.ky, p.idy) : p.idy * a; };
            double rhs[3];
            rhs[0] = mx(t.fx[0][r + 1][c] - t.fx[0][r][c]) - my(t.fy[0][r][c + 1] - t.fy[0][r][c]);
            rhs[1] = mx(t.fx[1][r + 1][c] - t.fx[2][r][c]) - my(t.fy[1][r][c + 1] - t.fy[1][r][c]);
            rhs[2] = mx(t.fx[3][r + 1][c] - t.fx[3][r][c]) - my(t.fy[2][r][c + 1] - t.fy[3][r][c]);
            const long long k = (long long)(i + NG) * p.P + (j + NG);
            const double *src[3] = {p.hs, p.hus, p.hvs}, *un[3] = {p.hn, p.hun, p.hvn};
            double o[3];
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                const double s = src[f][k];
                // 1.0 * s == s and 1.0 / 4.0 * s is an exponent shift, both exact
                if (p.stage == 1)
                    o[f] = s + cu(p.dt, rhs[f]);                                       // compute_U1
                else if (p.stage == 2)
                    o[f] = cu(3.0 / 4.0, un[f][k]) + x64::scale2(s, -2, 0.25) + cu(p.c2, rhs[f]);  // compute_U2
                else
                    o[f] = cu(1.0 / 3.0, un[f][k]) + cu(2.0 / 3.0, s) + cu(p.c3, rhs[f]);  // compute_U_next
            }
            if (BATHY) {  // enforce_positivity (serial_solver.hpp:453-478)
                if (x64::lt(o[0], H_FLOOR)) {
                    o[0] = H_FLOOR;
                    o[1] = 0.0;
                    o[2] = 0.0;
                }
                auto finite = [](double x) { return (x64::bits(x) & x64::ABS) < x64::INF_BITS; };
                bad = bad || !finite(o[0]) || !finite(o[1]) || !finite(o[2]);
            }
            p.ho[k] = o[0];
            p.huo[k] = o[1];
            p.hvo[k] = o[2];
        }
        if (kt + 1 < n_tiles) {
            __syncthreads();  // every update has read the x-interface rows
            for (int e = tid; e < 4 * TJ; e += NT) {
                const int q = e / TJ, cc = e - q * TJ;
                t.fx[q][0][cc] = t.fx[q][TI][cc];
            }
        }
    }
    if (bad) atomicOr(p.flags, FLAG_NONFINITE);
    if (fail) atomicOr(p.flags, FLAG_MODULAR_HLL);
}

// compute_stable_dt of time_utils.hpp:14-38 (the modular solver's CFL guard): the
// minimum over interior cells as the bit pattern of a non-negative double (the order of
// non-negative doubles), skipping NaN as std::min(dt_limit, NaN) keeps dt_limit; h < 0
// sets FLAG_NONFINITE, where the reference throws.
__global__ void k_modular_stable_dt(const double *h, const double *hu, const double *hv, int Nx,
                                    int Ny, long long P, double g, double cfl, double dx,
                                    double dy, unsigned long long *out, int *flags) {
    unsigned long long best = 0x7fefffffffffffffull;  // std::numeric_limits<double>::max()
    bool neg = false;
    const long long n = (long long)Nx * Ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / Ny), j = (int)(e - (e / Ny) * Ny);
        const long long k = (long long)(i + NG) * P + (j + NG);
        const double hh = h[k];
        if (hh < 0.0) neg = true;
        const double u = hu[k] / hh, v = hv[k] / hh;
        const double dt_cell = cfl / ((fabs(u) + sqrt(g * hh)) / dx + (fabs(v) + sqrt(g * hh)) / dy);
        if (dt_cell < __longlong_as_double((long long)best))
            best = (unsigned long long)__double_as_longlong(dt_cell);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other < best ? other : best;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(out, best);
    if (neg) atomicOr(flags, FLAG_NONFINITE);
}

static_assert(sizeof(Tile) <= 48 * 1024, "the tile fits the default shared-memory limit");

static int strip_tiles_mod(int tiles_j, int tile_rows) {
    if (SWE_MOD_STRIP > 0) return SWE_MOD_STRIP;
    static int sms[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) !=
                         cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    const long long waves16 = 16LL * SWE_MOD_MIN_BLOCKS * sms[dev];
    return (long long)tiles_j * ((tile_rows + 5) / 6) >= waves16 ? 6 : 1;
}

template <int RECON, int RIEMANN, bool BATHY>
cudaError_t launch_one(const ModParams &p, cudaStream_t s) {
    const int smem = (int)sizeof(Tile);
    const int tiles_j = (p.Ny + TJ - 1) / TJ, tile_rows = (p.Nx + TI - 1) / TI;
    const int strip = strip_tiles_mod(tiles_j, tile_rows);
    const dim3 grid(tiles_j, (tile_rows + strip - 1) / strip);
    k_modular_stage<RECON, RIEMANN, BATHY><<<grid, NT, smem, s>>>(p, strip);
    return cudaGetLastError();
}

template <int RECON, int RIEMANN>
cudaError_t launch_bathy(bool bathy, const ModParams &p, cudaStream_t s) {
    return bathy ? launch_one<RECON, RIEMANN, true>(p, s) : launch_one<RECON, RIEMANN, false>(p, s);
}

template <int RECON>
cudaError_t launch_riemann(int riemann, bool bathy, const ModParams &p, cudaStream_t s) {
    switch (riemann) {
        case 0: return launch_bathy<RECON, 0>(bathy, p, s);
        case 1: return launch_bathy<RECON, 1>(bathy, p, s);
        default: return launch_bathy<RECON, 2>(bathy, p, s);
    }
}

}  // namespace mod

cudaError_t launch_stage_modular(int stage, const ModularStage &m, cudaStream_t s) {
    mod::ModParams p;
    p.hs = static_cast<const double *>(m.hs);
    p.hus = static_cast<const double *>(m.hus);
    p.hvs = static_cast<const double *>(m.hvs);
    p.hn = static_cast<const double *>(m.hn);
    p.hun = static_cast<const double *>(m.hun);
    p.hvn = static_cast<const double *>(m.hvn);
    p.B = static_cast<const double *>(m.B);
    p.ho = static_cast<double *>(m.ho);
    p.huo = static_cast<double *>(m.huo);
    p.hvo = static_cast<double *>(m.hvo);
    p.Nx = m.Nx;
    p.Ny = m.Ny;
    p.P = m.pitch;
    p.g = m.g;
    p.half_g = 0.5 * m.g;
    p.nidx = -1.0 / m.dx;
    p.idy = 1.0 / m.dy;
    p.kx = m.kx;
    p.ky = m.ky;
    p.dt = m.dt;
    p.c2 = m.dt / 4.0;
    p.c3 = 2.0 * m.dt / 3.0;
    p.stage = stage;
    p.flags = m.flags;
    return m.recon == 0 ? mod::launch_riemann<0>(m.riemann, m.bathy != 0, p, s)
                        : mod::launch_riemann<1>(m.riemann, m.bathy != 0, p, s);
}

cudaError_t launch_modular_stable_dt(const void *h, const void *hu, const void *hv, int Nx, int Ny,
                                     long long pitch, double g, double cfl, double dx, double dy,
                                     unsigned long long *out, int *flags, int num_sms,
                                     cudaStream_t s) {
    const unsigned long long init = 0x7fefffffffffffffull;
    cudaError_t e = cudaMemcpyAsync(out, &init, sizeof init, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    const long long n = (long long)Nx * Ny;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 8ll * num_sms);
    mod::k_modular_stable_dt<<<blocks, 256, 0, s>>>(
        static_cast<const double *>(h), static_cast<const double *>(hu),
        static_cast<const double *>(hv), Nx, Ny, pitch, g, cfl, dx, dy, out, flags);
    return cudaGetLastError();
}

}  // namespace swe
