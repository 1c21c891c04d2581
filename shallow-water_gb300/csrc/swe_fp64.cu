// FP64 drop-in kernels: one fused kernel per SSP-RK3 stage.
//
// Bitwise parity with the reference's HPC_solver needs every floating-point
// operation of include/backend/serial/HPC/HPC_kernels.hpp in the same order and
// rounding: this translation unit is compiled with --fmad=false (no a*b+c fusion,
// which the reference's x86-64 Release build never does), double division and sqrt
// are IEEE round-to-nearest, and min/max are written as std::min/std::max.
//
// Stage kernel: a CTA owns a TI x TJ tile of interior cells.  It stages the tile plus
// a 2-cell halo of h, hu, hv, B (and eta = h + B) in shared memory, with the wall
// boundary condition applied through mirrored indices while loading, computes every
// x- and y-interface of the tile once, then each thread forms its cell's divergence
// (apply_divergence), the RK combine, positivity and the store.  Stage 3 also reduces
// the max wave speed of the new state (compute_stable_dt) into a device slot with a
// warp shuffle, a block reduction and one atomicMax per CTA.
//
// GB300 runs FP64 at ~2 operations/clock/SM, 1/64 of FP32, so the kernel is bound by
// the FP64 pipe, not by HBM.  Everything that need not be an FP64 instruction is moved
// to the integer pipe with bit-exact helpers (swe_f64_exact.cuh): compares, min/max,
// minmod's sign logic, positive parts, exact scalings by powers of two, and the
// reference's re-division (h*u)/h, which is decided from one exact FMA residual.
// Divisions and square roots, about twenty FP64-pipe slots each, are computed
// correctly rounded on the integer pipe (swe_soft_f64.cuh).
#include <algorithm>

#include "swe_common.cuh"
#include "swe_f64_exact.cuh"
#include "swe_soft_f64.cuh"
#include "swe_launch.h"
#include "swe_tma.cuh"

namespace swe {
namespace {

// Tile shapes are template parameters: TI rows (x) by TJ columns (y, contiguous),
// (TI + 1) * TJ threads, one per x-face (which also covers the TI * (TJ + 1) y-faces).

using x64::dmax;
using x64::dmin;

constexpr int64_t EPS_BITS = 0x3E45798EE2308C3ALL;  // bits of 1.0e-8
static_assert(sizeof(double) == 8, "double is binary64");

// safe_velocity (HPC_kernels.hpp:37-39), (h > 1e-8) ? q / h : 0.0, of two momenta over
// the same depth (one shared reciprocal).
__device__ __forceinline__ void safe_velocity2(double q1, double q2, double h, double &u1,
                                               double &u2) {
    if (x64::gt_pos_const(h, EPS_BITS)) {
        sf::div2_rn(q1, q2, h, u1, u2);
    } else {
        u1 = 0.0;
        u2 = 0.0;
    }
}

// Work split between the FP64 pipe and the integer pipes.  Each group of operations
// below runs either as FP64 instructions or as the correctly rounded integer routines
// of swe_soft_f64.cuh (identical results); moving part of the adds and multiplies off
// the FP64 pipe balances it against the integer pipes that carry the rest.
//   multiply groups: 0 momenta h*u, 1 physical fluxes, 2 HLL combination,
//                    3 wave-speed and bathymetry-correction products, 4 cell update;
//   add groups:      0 stencil differences, 1 reconstruction and depths, 2 wave
//                    speeds and flux sums, 3 HLL combination, 4 corrections and
//                    cell update.
#ifndef SWE_F64_SOFT_MUL
#define SWE_F64_SOFT_MUL 0x00
#endif
#ifndef SWE_F64_SOFT_ADD
#define SWE_F64_SOFT_ADD 0x00
#endif

template <int G>
__device__ __forceinline__ double fmul(double a, double b) {
    if constexpr (((SWE_F64_SOFT_MUL) >> G) & 1) return sf::mul_rn(a, b);
    else return a * b;
}
template <int G>
__device__ __forceinline__ double fadd(double a, double b) {
    if constexpr (((SWE_F64_SOFT_ADD) >> G) & 1) return sf::add_rn(a, b);
    else return a + b;
}
template <int G>
__device__ __forceinline__ double fsub(double a, double b) {
    if constexpr (((SWE_F64_SOFT_ADD) >> G) & 1) return sf::sub_rn(a, b);
    else return a - b;
}

// The cell update's products (dt x L, the RK weights, 1/dx when it is not a power of
// two): on the integer pipes when SOFT.  The single-grid stage kernel is 0.8% faster
// with them there; the ensemble kernel is not (see the kernels below).
template <bool SOFT>
__device__ __forceinline__ double cu_mul(double a, double b) {
    if constexpr (SOFT) return sf::mul_rn(a, b);
    else return fmul<4>(a, b);
}

// Exact multiplication by a grid constant that may be a power of two (k != 127).
template <bool SOFT>
__device__ __forceinline__ double mul_const(double c, int k, double x) {
    return k != 127 ? x64::scale2(x, k, c) : cu_mul<SOFT>(c, x);
}

// hll_x (HPC_kernels.hpp:46-82) in normal/tangential form; hll_y (:84-120) is the
// same with hv normal and hu tangential.  The left/right states are
// (hL, hL*unm, hL*utm) and (hR, hR*unp, hR*utp) as built at :164-169; the velocities
// the reference recomputes from them, (hL*unm)/hL etc., come from x64::redivide.
__device__ __forceinline__ void hll_normal(double g, double half_g, double hL, double unm,
                                           double utm, double hR, double unp, double utp,
                                           double &fh, double &fqn, double &fqt) {
    const double qnL = fmul<0>(hL, unm), qtL = fmul<0>(hL, utm);
    const double qnR = fmul<0>(hR, unp), qtR = fmul<0>(hR, utp);
    const bool wetL = x64::gt_pos_const(hL, EPS_BITS), wetR = x64::gt_pos_const(hR, EPS_BITS);
    const double unL = wetL ? x64::redivide(qnL, hL, unm) : 0.0;
    const double utL = wetL ? x64::redivide(qtL, hL, utm) : 0.0;
    const double unR = wetR ? x64::redivide(qnR, hR, unp) : 0.0;
    const double utR = wetR ? x64::redivide(qtR, hR, utp) : 0.0;
    // Wave speeds of both sides through one inlined copy of the square root.
    double cL = 0.0, cR = 0.0;
#pragma unroll 1
    for (int side = 0; side < 2; ++side) {
        const double c = sf::sqrt_rn(fmul<3>(g, side ? hR : hL));
        if (side)
            cR = c;
        else
            cL = c;
    }
    const double sL = dmin(fsub<2>(unL, cL), fsub<2>(unR, cR));
    const double sR = dmax(fadd<2>(unL, cL), fadd<2>(unR, cR));
    const double FL_h = qnL;
    const double FL_n = fadd<2>(fmul<1>(qnL, unL), fmul<1>(fmul<1>(half_g, hL), hL));
    const double FL_t = fmul<1>(qnL, utL);
    const double FR_h = qnR;
    const double FR_n = fadd<2>(fmul<1>(qnR, unR), fmul<1>(fmul<1>(half_g, hR), hR));
    const double FR_t = fmul<1>(qnR, utR);
    if (x64::le(0.0, sL)) {
        fh = FL_h;
        fqn = FL_n;
        fqt = FL_t;
    } else if (x64::le(sR, 0.0)) {
        fh = FR_h;
        fqn = FR_n;
        fqt = FR_t;
    } else {
        // (sR*FL - sL*FR + sL*sR*(UR - UL)) / (sR - sL), the division as a product with
        // the reciprocal exactly as the reference writes it
        const double inv = sf::div_rn(1.0, fsub<3>(sR, sL));
        const double sLsR = fmul<2>(sL, sR);
        fh = fmul<2>(fadd<3>(fsub<3>(fmul<2>(sR, FL_h), fmul<2>(sL, FR_h)),
                             fmul<2>(sLsR, fsub<3>(hR, hL))),
                     inv);
        fqn = fmul<2>(fadd<3>(fsub<3>(fmul<2>(sR, FL_n), fmul<2>(sL, FR_n)),
                              fmul<2>(sLsR, fsub<3>(qnR, qnL))),
                      inv);
        fqt = fmul<2>(fadd<3>(fsub<3>(fmul<2>(sR, FL_t), fmul<2>(sL, FR_t)),
                              fmul<2>(sLsR, fsub<3>(qtR, qtL))),
                      inv);
    }
}

// One interface between stencil cells m1, c0 (minus side), p1 (plus side), p2, as
// in compute_x_fluxes (HPC_kernels.hpp:136-184) / compute_y_fluxes (:203-251).
// qn: normal momentum, qt: tangential.  eta values are h + B of the same cells.
struct Face {
    double fh, fqt, fqn_m, fqn_p;
};

// The stencil differences (d0 = x0 - x_m1, d1 = x_p1 - x0, d2 = x_p2 - x_p1 of eta, qn,
// qt) are computed once per cell pair in shared memory and shared by the three
// interfaces that use each of them; the values are the reference's own differences.
__device__ __forceinline__ Face face_flux(double g, double half_g, double eta_0, double eta_p1,
                                          double d_eta0, double d_eta1, double d_eta2,
                                          double qn_0, double qn_p1, double d_qn0,
                                          double d_qn1, double d_qn2, double qt_0,
                                          double qt_p1, double d_qt0, double d_qt1,
                                          double d_qt2, double b_minus, double b_plus) {
    const double eta_minus = fadd<1>(eta_0, x64::halve(x64::minmod(d_eta0, d_eta1)));
    const double eta_plus = fsub<1>(eta_p1, x64::halve(x64::minmod(d_eta1, d_eta2)));
    const double qn_minus = fadd<1>(qn_0, x64::halve(x64::minmod(d_qn0, d_qn1)));
    const double qt_minus = fadd<1>(qt_0, x64::halve(x64::minmod(d_qt0, d_qt1)));
    const double qn_plus = fsub<1>(qn_p1, x64::halve(x64::minmod(d_qn1, d_qn2)));
    const double qt_plus = fsub<1>(qt_p1, x64::halve(x64::minmod(d_qt1, d_qt2)));
    // b_star = std::max(b_minus, b_plus) is bitwise one of them: on that side
    // hs = positive(eta - b_star) is h itself and corr = half_g * (h*h - h*h) is +0, so
    // only the other side's hs and correction are computed (the same operations as the
    // reference's on that side); f_n + (+0) is f_n with -0 turned into +0.
    const bool m_star = !x64::lt(b_minus, b_plus);
    const double b_star = m_star ? b_minus : b_plus;
    const double h_minus = x64::positive_part(fsub<1>(eta_minus, b_minus));
    const double h_plus = x64::positive_part(fsub<1>(eta_plus, b_plus));
    // Velocities of both sides through one inlined copy of the division.
    double un_minus = 0.0, ut_minus = 0.0, un_plus = 0.0, ut_plus = 0.0;
#pragma unroll 1
    for (int side = 0; side < 2; ++side) {
        double a, b;
        safe_velocity2(side ? qn_plus : qn_minus, side ? qt_plus : qt_minus,
                       side ? h_plus : h_minus, a, b);
        if (side) {
            un_plus = a;
            ut_plus = b;
        } else {
            un_minus = a;
            ut_minus = b;
        }
    }
    const double h_o = m_star ? h_plus : h_minus;  // the side b_star is not taken from
    const double hs_o = x64::positive_part(fsub<1>(m_star ? eta_plus : eta_minus, b_star));
    const double hs_minus = m_star ? h_minus : hs_o;
    const double hs_plus = m_star ? hs_o : h_plus;
    double f_h, f_n, f_t;
    hll_normal(g, half_g, hs_minus, un_minus, ut_minus, hs_plus, un_plus, ut_plus, f_h, f_n,
               f_t);
    const double corr_o = fmul<3>(half_g, fsub<4>(fmul<3>(h_o, h_o), fmul<3>(hs_o, hs_o)));
    const double fqn_o = fadd<4>(f_n, corr_o);
    const double fqn_s = x64::bits(f_n) == x64::SIGN ? 0.0 : f_n;
    Face f;
    f.fh = f_h;
    f.fqt = f_t;
    f.fqn_m = m_star ? fqn_s : fqn_o;
    f.fqn_p = m_star ? fqn_o : fqn_s;
    return f;
}

// Per-cell wave speed max(|u| + c, |v| + c) (compute_stable_dt body, :288-293), as
// max(|hu|, |hv|) / h + c.  Correct rounding is monotonic, so for finite values
// fl(max(a, b) / h) = max(fl(a / h), fl(b / h)) and fl(m + c) = max(fl(|u| + c),
// fl(|v| + c)): the same bits with one division and one add instead of two each.  (A
// non-finite state fails the step in the same kernel, whatever its speed.)
__device__ __forceinline__ double cell_speed(double g, double h, double hu, double hv) {
    const double m = x64::gt_pos_const(h, EPS_BITS)
                         ? sf::div_rn(dmax(x64::fabs_(hu), x64::fabs_(hv)), h) : 0.0;
    const double c = sf::sqrt_rn(g * x64::positive_part(h));  // std::max(0.0, h)
    return m + c;
}

// Block max of per-thread non-negative speeds, then one atomicMax on the bit pattern
// (order-preserving for non-negative doubles).
__device__ __forceinline__ void block_max_to_slot(double v, unsigned long long *slot) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0) atomicMax(slot, (unsigned long long)__double_as_longlong(v));
    }
}

// The step's dt (compute_stable_dt, HPC_kernels.hpp:296-297, on the max speed reduced by
// the previous step), computed once per block and shared.  `abort` is true
// (block-uniform) when FLAG_TIMEOUT is already set, read under the same barrier; STAGE 0
// (no dt) only reads the flag.
template <bool DT = true>
__device__ __forceinline__ double stage_dt(const StageParams &p, bool &abort) {
    __shared__ double s_dt;
    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        double dt = p.dt_fixed;
        if (DT && !(dt > 0.0)) {
            const double ms = __longlong_as_double((long long)p.speed[p.slot_read]);
            dt = x64::le(ms, EPS) ? 1.0e100 : p.cfl_min_dxdy / ms;
        }
        s_dt = dt;
        s_abort = tma::timeout_set(p.flags);
    }
    __syncthreads();
    abort = s_abort != 0;
    return s_dt;
}
__device__ __forceinline__ double stage_dt(const StageParams &p) {
    bool abort;
    return stage_dt<true>(p, abort);
}

// One tile of one RK stage: stage the TI x TJ tile (origin i0, j0 in interior
// coordinates) plus a 2-cell halo, compute its interfaces, and update its cells.
// Returns the thread's cell wave speed of the new state (stage 3), else 0.
// (TI + 1) * TJ threads; the caller provides dt (same for the whole block).
// Shared memory of one tile (dynamic: up to 53 KB for the 4x64 shape).
template <int TI, int TJ>
struct TileF64 {
    static constexpr int RI = TI + 4, RJ = TJ + 4;
    double hu[RI][RJ], hv[RI][RJ], B[RI][RJ], eta[RI][RJ];  // tile + 2-cell halo
    double dx[3][RI - 1][TJ];  // eta, hu, hv: row r minus row r - 1 (r = 1..RI-1), tile columns
    double dy[3][TI][RJ - 1];  // eta, hu, hv: column c minus column c - 1, tile rows
    double xf[4][TI + 1][TJ];  // x-interfaces: fh, fhv, fhu_m, fhu_p
    double yf[4][TI][TJ + 1];  // y-interfaces: gh, ghu, ghv_m, ghv_p
    uint64_t bar;              // TMA transaction barrier
};
// The halo arrays are multiples of 128 bytes, so with the struct 128-byte aligned every
// TMA destination is too.
static_assert(sizeof(double) * (8 + 4) * (32 + 4) % 128 == 0, "TMA destinations aligned");

template <int TI, int TJ>
__device__ __forceinline__ TileF64<TI, TJ> &tile_smem() {
    extern __shared__ unsigned char smem_f64[];  // sizeof(TileF64) + 128 bytes
    const uint32_t a = tma::smem_u32(smem_f64);
    return *reinterpret_cast<TileF64<TI, TJ> *>(smem_f64 + ((128u - (a & 127u)) & 127u));
}

// One tile of one RK stage: stage the TI x TJ tile (origin i0, j0 in interior
// coordinates) plus a 2-cell halo, compute its interfaces, and update its cells.
// Returns the thread's cell wave speed of the new state (stage 3), else 0.
// (TI + 1) * TJ threads; the caller provides dt (same for the whole block).
// Interior tiles are staged by TMA through `pipe` when tm is given; `aborted` is set
// (block-uniform) when that wait gave up, and the caller then returns from the kernel.
// carry_in: the tile's first x-face row (between tile rows -1 and 0) is already in
// xf[.][0] - the previous tile of the strip computed it as its last row - and is not
// recomputed.  carry_out: after the update, the tile's last x-face row is moved to
// xf[.][0] for the next tile of the strip.
template <int TI, int TJ, int STAGE, bool SOFT_CU>
__device__ __forceinline__ double stage_tile_f64(const StageParams &p, int i0, int j0,
                                                 double dt, const tma::TileMaps *tm,
                                                 tma::Pipe &pipe, bool &aborted,
                                                 bool carry_in = false, bool carry_out = false) {
    constexpr int NT = (TI + 1) * TJ, RI = TI + 4, RJ = TJ + 4;
    static_assert(TI * (TJ + 1) <= NT, "one thread per y-face");
    TileF64<TI, TJ> &S = tile_smem<TI, TJ>();

    const int tid = threadIdx.x;
    const long long P = p.pitch;
    const double *hs = static_cast<const double *>(p.hs);
    const double *hus = static_cast<const double *>(p.hus);
    const double *hvs = static_cast<const double *>(p.hvs);
    const double *Bg = static_cast<const double *>(p.B);

    // Stage the tile + halo.  Tiles whose halo lies inside the interior are copied by
    // TMA (h lands in eta and becomes h + B in place); tiles that touch a wall or a slab
    // interface read through mirrored indices, ghosts from the wall rule.
    const bool interior = tm != nullptr && i0 >= NG && j0 >= NG && i0 + TI + NG <= p.Nx &&
                          j0 + TJ + NG <= p.Ny;
    aborted = false;
    if (interior) {
        // halo origin (i0 - 2, j0 - 2) in interior coordinates = (i0, j0) in the ghosted
        // array; j0 is a multiple of TJ, so x * 8 bytes is 16-byte aligned
        uint64_t *bar = pipe.bar;
        if (!tma::stage_in(pipe, p.flags, 4u * RI * RJ * sizeof(double), [&] {
                tma::load_2d(&S.eta[0][0], tm->e, j0, i0, bar);
                tma::load_2d(&S.hu[0][0], tm->u, j0, i0, bar);
                tma::load_2d(&S.hv[0][0], tm->v, j0, i0, bar);
                tma::load_2d(&S.B[0][0], tm->b, j0, i0, bar);
            })) {
            aborted = true;
            return 0.0;
        }
        for (int t = tid; t < RI * RJ; t += NT) {
            const int r = t / RJ, c = t - (t / RJ) * RJ;
            S.eta[r][c] = S.eta[r][c] + S.B[r][c];  // h + B
        }
    } else {
        for (int t = tid; t < RI * RJ; t += NT) {
            const int r = t / RJ, c = t - (t / RJ) * RJ;
            const int ii = i0 - NG + r, jj = j0 - NG + c;
            bool fx, fy;
            const int mi = map_row(ii, p.Nx, p.bc, p.halo_lo, p.halo_hi, fx);
            const int mj = map_coord(jj, p.Ny, p.bc, fy);
            const long long k = (long long)(mi + NG) * P + (mj + NG);
            const double hv_ = hvs[k], hu_ = hus[k], h_ = hs[k];
            // B is read where it lies, ghosts included (clamped in overhanging tiles).
            const int bi = clamp_int(ii + NG, 0, p.Nx + 2 * NG - 1);
            const int bj = clamp_int(jj + NG, 0, p.Ny + 2 * NG - 1);
            const double b_ = Bg[(long long)bi * P + bj];
            S.hu[r][c] = fx ? x64::neg(hu_) : hu_;
            S.hv[r][c] = fy ? x64::neg(hv_) : hv_;
            S.B[r][c] = b_;
            S.eta[r][c] = h_ + b_;
        }
    }
    __syncthreads();

    // Stencil differences: x along the tile columns, y along the tile rows.
    constexpr int NDX = (RI - 1) * TJ, NDY = TI * (RJ - 1);
    for (int t = tid; t < NDX + NDY; t += NT) {
        if (t < NDX) {
            const int r = t / TJ + 1, c = t - (t / TJ) * TJ;
            S.dx[0][r - 1][c] = S.eta[r][c + NG] - S.eta[r - 1][c + NG];
            S.dx[1][r - 1][c] = S.hu[r][c + NG] - S.hu[r - 1][c + NG];
            S.dx[2][r - 1][c] = S.hv[r][c + NG] - S.hv[r - 1][c + NG];
        } else {
            const int u = t - NDX;
            const int r = u / (RJ - 1), c = u - (u / (RJ - 1)) * (RJ - 1) + 1;
            S.dy[0][r][c - 1] = S.eta[r + NG][c] - S.eta[r + NG][c - 1];
            S.dy[1][r][c - 1] = S.hu[r + NG][c] - S.hu[r + NG][c - 1];
            S.dy[2][r][c - 1] = S.hv[r + NG][c] - S.hv[r + NG][c - 1];
        }
    }
    __syncthreads();

    const double g = p.g, half_g = p.half_g;
    // Interfaces, one code path for both directions (a single inlined copy of the flux
    // keeps the kernel within the instruction cache):
    //  pass 0, x-faces between tile rows a = fr + 1 and a + 1, fr in [0, TI], one per
    //    thread; the difference of rows a and a - 1 is dx[.][fr];
    //  pass 1, y-faces between tile columns a = fc + 1 and a + 1, fc in [0, TJ]; the
    //    difference of columns a and a - 1 is dy[.][fr][fc].
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
        const bool xp = pass == 0;
        if (!xp && tid >= TI * (TJ + 1)) break;
        if (xp && carry_in && tid < TJ) continue;  // x-face row 0 came from the last tile
        const int W = xp ? TJ : TJ + 1;
        const int fr = tid / W, fc = tid - (tid / W) * W;
        // cells c0 and p1 of the stencil and the three differences of each field
        const int r0 = xp ? fr + 1 : fr + NG, c0 = xp ? fc + NG : fc + 1;
        const int r1 = xp ? r0 + 1 : r0, c1 = xp ? c0 : c0 + 1;
        const double *D0 = xp ? &S.dx[0][fr][fc] : &S.dy[0][fr][fc];
        const double *Dn = xp ? &S.dx[1][fr][fc] : &S.dy[2][fr][fc];  // normal momentum
        const double *Dt = xp ? &S.dx[2][fr][fc] : &S.dy[1][fr][fc];  // tangential
        const int st = xp ? TJ : 1;  // stride to the next difference
        const double(*N)[TileF64<TI, TJ>::RJ] = xp ? S.hu : S.hv;
        const double(*T)[TileF64<TI, TJ>::RJ] = xp ? S.hv : S.hu;
        const Face F = face_flux(g, half_g, S.eta[r0][c0], S.eta[r1][c1], D0[0], D0[st],
                                 D0[2 * st], N[r0][c0], N[r1][c1], Dn[0], Dn[st], Dn[2 * st],
                                 T[r0][c0], T[r1][c1], Dt[0], Dt[st], Dt[2 * st], S.B[r0][c0],
                                 S.B[r1][c1]);
        if (xp) {
            S.xf[0][fr][fc] = F.fh;
            S.xf[1][fr][fc] = F.fqt;
            S.xf[2][fr][fc] = F.fqn_m;
            S.xf[3][fr][fc] = F.fqn_p;
        } else {
            S.yf[0][fr][fc] = F.fh;
            S.yf[1][fr][fc] = F.fqt;
            S.yf[2][fr][fc] = F.fqn_m;
            S.yf[3][fr][fc] = F.fqn_p;
        }
    }
    __syncthreads();

    const int ty = tid / TJ, tx = tid - (tid / TJ) * TJ;
    const int ii = i0 + ty, jj = j0 + tx;
    const bool inside = (ty < TI) && (ii < p.Nx) && (jj < p.Ny);
    double speed = 0.0;
    if (inside) {
        // apply_divergence (HPC_kernels.hpp:274-276): right/top face minus-side
        // fluxes against left/bottom face plus-side fluxes.
        // -inv_dx * (a - b) - inv_dy * (c - d); (-c) * x == -(c * x) exactly.
        const double rh =
            fsub<4>(x64::neg(mul_const<SOFT_CU>(p.inv_dx, p.kx, fsub<4>(S.xf[0][ty + 1][tx], S.xf[0][ty][tx]))),
                    mul_const<SOFT_CU>(p.inv_dy, p.ky, fsub<4>(S.yf[0][ty][tx + 1], S.yf[0][ty][tx])));
        const double rhu =
            fsub<4>(x64::neg(mul_const<SOFT_CU>(p.inv_dx, p.kx, fsub<4>(S.xf[2][ty + 1][tx], S.xf[3][ty][tx]))),
                    mul_const<SOFT_CU>(p.inv_dy, p.ky, fsub<4>(S.yf[1][ty][tx + 1], S.yf[1][ty][tx])));
        const double rhv =
            fsub<4>(x64::neg(mul_const<SOFT_CU>(p.inv_dx, p.kx, fsub<4>(S.xf[1][ty + 1][tx], S.xf[1][ty][tx]))),
                    mul_const<SOFT_CU>(p.inv_dy, p.ky, fsub<4>(S.yf[2][ty][tx + 1], S.yf[3][ty][tx])));
        const long long k = (long long)(ii + NG) * P + (jj + NG);
        if constexpr (STAGE == 0) {  // L(U^n) alone: stage 1 before its dt is known
            static_cast<double *>(p.ho)[k] = rh;
            static_cast<double *>(p.huo)[k] = rhu;
            static_cast<double *>(p.hvo)[k] = rhv;
        } else {
            const double sh = hs[k];  // interior cell: no ghost mapping
            const double shu = S.hu[ty + NG][tx + NG];
            const double shv = S.hv[ty + NG][tx + NG];
            // U + dt * L(U)
            const double eh = fadd<4>(sh, cu_mul<SOFT_CU>(dt, rh));
            const double ehu = fadd<4>(shu, cu_mul<SOFT_CU>(dt, rhu));
            const double ehv = fadd<4>(shv, cu_mul<SOFT_CU>(dt, rhv));
            double oh, ohu, ohv;
            if (STAGE == 1) {  // HPC_solver.hpp:246-248
                oh = eh;
                ohu = ehu;
                ohv = ehv;
            } else {
                const double nh = static_cast<const double *>(p.hn)[k];
                const double nhu = static_cast<const double *>(p.hun)[k];
                const double nhv = static_cast<const double *>(p.hvn)[k];
                if (STAGE == 2) {  // HPC_solver.hpp:271-273
                    oh = fadd<4>(cu_mul<SOFT_CU>(0.75, nh), x64::scale2(eh, -2, 0.25));
                    ohu = fadd<4>(cu_mul<SOFT_CU>(0.75, nhu), x64::scale2(ehu, -2, 0.25));
                    ohv = fadd<4>(cu_mul<SOFT_CU>(0.75, nhv), x64::scale2(ehv, -2, 0.25));
                } else {  // HPC_solver.hpp:296-300
                    oh = fadd<4>(cu_mul<SOFT_CU>(1.0 / 3.0, nh), cu_mul<SOFT_CU>(2.0 / 3.0, eh));
                    ohu = fadd<4>(cu_mul<SOFT_CU>(1.0 / 3.0, nhu), cu_mul<SOFT_CU>(2.0 / 3.0, ehu));
                    ohv = fadd<4>(cu_mul<SOFT_CU>(1.0 / 3.0, nhv), cu_mul<SOFT_CU>(2.0 / 3.0, ehv));
                }
            }
            // enforce_positivity (HPC_kernels.hpp:305-312)
            const bool clamped = x64::lt(oh, H_FLOOR);
            if (clamped) {
                oh = H_FLOOR;
                ohu = 0.0;
                ohv = 0.0;
            }
            if (p.mask) p.mask[k] = clamped ? 1 : 0;
            if (((x64::bits(oh) & x64::ABS) >= x64::INF_BITS) ||
                ((x64::bits(ohu) & x64::ABS) >= x64::INF_BITS) ||
                ((x64::bits(ohv) & x64::ABS) >= x64::INF_BITS))
                atomicOr(p.flags, FLAG_NONFINITE);
            static_cast<double *>(p.ho)[k] = oh;
            static_cast<double *>(p.huo)[k] = ohu;
            static_cast<double *>(p.hvo)[k] = ohv;
            if (STAGE == 3) speed = cell_speed(g, oh, ohu, ohv);
        }
    }
    if (carry_out) {
        // Every update has read x-face row 0 (the barrier); the next tile's first row is
        // this tile's last.  Its staging touches only the halo arrays, and barriers
        // order this copy before its x-face pass.
        __syncthreads();
        for (int t = tid; t < 4 * TJ; t += NT) {
            const int f = t / TJ, c = t - (t / TJ) * TJ;
            S.xf[f][0][c] = S.xf[f][TI][c];
        }
    }
    return speed;
}

// Resident threads per SM the register budget is sized for: 1152 (36 warps, four
// 8x32 tiles) keeps the FP64 pipe fed while other CTAs load or synchronise.
#ifndef SWE_F64_THREADS_PER_SM
#define SWE_F64_THREADS_PER_SM 1152
#endif
#ifndef SWE_ENS_F64_THREADS_PER_SM
#define SWE_ENS_F64_THREADS_PER_SM 1152
#endif
#ifndef SWE_ENS_F64_SOFT_CU
#define SWE_ENS_F64_SOFT_CU 0
#endif
constexpr int min_blocks(int TI, int TJ) {
    return SWE_F64_THREADS_PER_SM / ((TI + 1) * TJ) > 0 ? SWE_F64_THREADS_PER_SM / ((TI + 1) * TJ) : 1;
}
constexpr int ens_min_blocks(int TI, int TJ) {
    return SWE_ENS_F64_THREADS_PER_SM / ((TI + 1) * TJ) > 0
               ? SWE_ENS_F64_THREADS_PER_SM / ((TI + 1) * TJ) : 1;
}

// Tiles per CTA of the single-grid stage kernel: a CTA walks a strip of this many tiles
// along x and carries each tile's last x-face row into the next, so that only one x-face
// row in a strip is computed twice: 2.05 interfaces per cell for 6 tiles, against 2.16
// for lone 8x32 tiles.  Fewer, longer CTAs fill the GPU less evenly, so the length is
// chosen per grid (strip_tiles_f64): six tiles while they leave at least 16 waves of
// resident CTAs, else four under the same rule, else lone tiles.  Measured (GCUPS, the
// same bits for every length):
//   8192^2: lone 1.043-1.046, 2 1.032, 3 1.050, 4 1.056-1.058, 5 1.057, 6 1.061-1.062,
//           7 1.054, 8 1.053, 16 1.052;
//   4096^2: lone 1.040, 2 1.029, 4 1.048, 6 1.050;
//   2048^2: lone 1.029, 2 1.018, 4 1.025, 6 1.015;
//   1024^2: lone 1.001, 2 0.962, 4 0.948, 6 0.864.
// SWE_F64_STRIP > 0 fixes the length instead.
#ifndef SWE_F64_STRIP
#define SWE_F64_STRIP 0
#endif

// Single grid: CTA (blockIdx.x, blockIdx.y) owns tile column blockIdx.x of the strip of
// tile rows [p.tile_row0 + blockIdx.y * STRIP, ...), clipped to [p.tile_row0, tile_row1).
// STAGE 0 is stage 1 without its dt: it stores L(U^n) in the output buffers, and
// k_combine1_f64 forms U^(1) once the max wave speed is reduced.
template <int TI, int TJ, int STAGE>
__global__ void __launch_bounds__((TI + 1) * TJ, min_blocks(TI, TJ))
    k_stage_f64(const StageParams p, const __grid_constant__ CUtensorMap tm_h,
                const __grid_constant__ CUtensorMap tm_u,
                const __grid_constant__ CUtensorMap tm_v,
                const __grid_constant__ CUtensorMap tm_b, int use_tma, int tile_row1,
                int strip) {
    TileF64<TI, TJ> &S = tile_smem<TI, TJ>();
    if (use_tma && threadIdx.x == 0) tma::mbar_init(&S.bar, 1);  // visible after stage_dt
    bool aborted;
    const double dt = stage_dt<STAGE != 0>(p, aborted);
    if (aborted) return;  // an earlier wait of this call gave up
    const tma::TileMaps maps{&tm_h, &tm_u, &tm_v, &tm_b};
    tma::Pipe pipe{&S.bar, 0u};
    const int tr0 = p.tile_row0 + (int)blockIdx.y * strip;
    const int n = min(strip, tile_row1 - tr0);
    double speed = 0.0;
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        const double v = stage_tile_f64<TI, TJ, STAGE, true>(
            p, (tr0 + k) * TI, blockIdx.x * TJ, dt, use_tma ? &maps : nullptr, pipe, aborted,
            k > 0, k + 1 < n);
        if (aborted) return;
        if constexpr (STAGE == 3) speed = dmax(speed, v);
    }
    const bool first = blockIdx.x == 0 && tr0 == 0 && threadIdx.x == 0;
    if (STAGE == 1 && first) {
        p.speed[p.slot_write] = 0ull;  // read by nobody until stage 3 of this step
        if (p.dt_log) p.dt_log[p.log_index] = dt;
    }
    if (STAGE == 3) {
        block_max_to_slot(speed, p.speed + p.slot_write);
        if (first && p.t_accum) *p.t_accum += dt;
    }
}

// The rest of stage 1 after k_stage_f64<.., 0>: U^(1) = U^n + dt L(U^n) with the
// positivity correction and the non-finite check, the same operations in the same
// order as the fused stage (HPC_solver.hpp:246-248, HPC_kernels.hpp:305-312).
// p.ho/huo/hvo hold L on entry (read) and receive U^(1) through (o_h, o_hu, o_hv).
__global__ void __launch_bounds__(256) k_combine1_f64(const StageParams p, double *o_h,
                                                      double *o_hu, double *o_hv) {
    const double dt = stage_dt(p);
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        p.speed[p.slot_write] = 0ull;
        if (p.dt_log) p.dt_log[p.log_index] = dt;
    }
    const double *hs = static_cast<const double *>(p.hs);
    const double *hus = static_cast<const double *>(p.hus);
    const double *hvs = static_cast<const double *>(p.hvs);
    const double *lh = static_cast<const double *>(p.ho);
    const double *lhu = static_cast<const double *>(p.huo);
    const double *lhv = static_cast<const double *>(p.hvo);
    bool bad = false;
    for (int i = blockIdx.y; i < p.Nx; i += gridDim.y)
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < p.Ny; j += gridDim.x * blockDim.x) {
        const long long k = (long long)(i + NG) * p.pitch + (j + NG);
        double oh = fadd<4>(hs[k], cu_mul<true>(dt, lh[k]));
        double ohu = fadd<4>(hus[k], cu_mul<true>(dt, lhu[k]));
        double ohv = fadd<4>(hvs[k], cu_mul<true>(dt, lhv[k]));
        const bool clamped = x64::lt(oh, H_FLOOR);
        if (clamped) {
            oh = H_FLOOR;
            ohu = 0.0;
            ohv = 0.0;
        }
        if (p.mask) p.mask[k] = clamped ? 1 : 0;
        bad |= ((x64::bits(oh) & x64::ABS) >= x64::INF_BITS) ||
               ((x64::bits(ohu) & x64::ABS) >= x64::INF_BITS) ||
               ((x64::bits(ohv) & x64::ABS) >= x64::INF_BITS);
        o_h[k] = oh;
        o_hu[k] = ohu;
        o_hv[k] = ohv;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(p.flags, FLAG_NONFINITE);
}

// Ensemble: CTAs stride over a flat list of (instance, tile) work items; every tile
// costs the same, so static striding balances.  Each instance has its own dt, max-speed
// slots and time (per-instance CFL).
template <int TI, int TJ, int STAGE>
__global__ void __launch_bounds__((TI + 1) * TJ, ens_min_blocks(TI, TJ)) k_ens_stage_f64(const EnsParams e) {
    // The instance's view lives in shared memory, read where used (see k_ens_stage_f32).
    __shared__ StageParams s_p;
    __shared__ int s_t;
    tma::Pipe pipe{nullptr, 0u};  // no TMA: every tile uses the mirrored-index loader
    for (int T = blockIdx.x; T < e.total_tiles; T += gridDim.x) {
        if (threadIdx.x == 0) {
            const int q = e.tile_inst[T];
            s_p = ens_view(e, q);
            s_t = T - e.inst[q].tile_base;
        }
        __syncthreads();
        const StageParams &p = s_p;
        const int q = e.tile_inst[T];
        const int t = s_t;
        const int tiles_j = e.inst[q].tiles_j;
        const int ti = t / tiles_j, tj = t - (t / tiles_j) * tiles_j;
        bool aborted;
        const double dt = stage_dt<true>(p, aborted);
        if (aborted) return;  // FLAG_TIMEOUT set: the call has failed, the launch ends
        const double speed = stage_tile_f64<TI, TJ, STAGE, SWE_ENS_F64_SOFT_CU != 0>(
            p, ti * TI, tj * TJ, dt, nullptr, pipe, aborted);
        if (STAGE == 1 && t == 0 && threadIdx.x == 0) {
            p.speed[p.slot_write] = 0ull;
            if (e.dt_last) e.dt_last[q] = dt;
        }
        if (STAGE == 3) {
            block_max_to_slot(speed, p.speed + p.slot_write);
            if (t == 0 && threadIdx.x == 0) e.t[q] += dt;
        }
        __syncthreads();  // the next tile reuses the shared tile buffers
    }
}

// SHAPE_STRIP: a work item is a strip of up to F64_STRIP_TILES 8x32 tiles along x of one
// instance, walked as the single-grid kernel walks its strips (the last x-face row of a
// tile carried into the next); the same schedule and per-instance duties as
// k_ens_stage_f64.
template <int STAGE>
__global__ void __launch_bounds__(9 * 32, ens_min_blocks(8, 32)) k_ens_stage_f64_strip(const EnsParams e) {
    __shared__ StageParams s_p;
    __shared__ int s_t;
    tma::Pipe pipe{nullptr, 0u};  // no TMA: every tile uses the mirrored-index loader
    for (int T = blockIdx.x; T < e.total_tiles; T += gridDim.x) {
        if (threadIdx.x == 0) {
            const int q = e.tile_inst[T];
            s_p = ens_view(e, q);
            s_t = T - e.inst[q].tile_base;
        }
        __syncthreads();
        const StageParams &p = s_p;
        const int q = e.tile_inst[T];
        const int t = s_t;
        const int tiles_j = e.inst[q].tiles_j;
        const int si = t / tiles_j, tj = t - (t / tiles_j) * tiles_j;
        const int tr0 = si * F64_STRIP_TILES;
        const int n = min(F64_STRIP_TILES, (p.Nx + 7) / 8 - tr0);
        bool aborted;
        const double dt = stage_dt<true>(p, aborted);
        if (aborted) return;  // FLAG_TIMEOUT set: the call has failed, the launch ends
        double speed = 0.0;
#pragma unroll 1
        for (int k = 0; k < n; ++k) {
            const double v = stage_tile_f64<8, 32, STAGE, SWE_ENS_F64_SOFT_CU != 0>(
                p, (tr0 + k) * 8, tj * 32, dt, nullptr, pipe, aborted, k > 0, k + 1 < n);
            if constexpr (STAGE == 3) speed = dmax(speed, v);
        }
        if (STAGE == 1 && t == 0 && threadIdx.x == 0) {
            p.speed[p.slot_write] = 0ull;
            if (e.dt_last) e.dt_last[q] = dt;
        }
        if (STAGE == 3) {
            block_max_to_slot(speed, p.speed + p.slot_write);
            if (t == 0 && threadIdx.x == 0) e.t[q] += dt;
        }
        __syncthreads();  // the next item reuses the shared tile buffers
    }
}

// Max wave speed of interior rows [i0, i1) of a state into one slot (after an upload,
// whole or by bands of rows).
__global__ void __launch_bounds__(256) k_max_speed_f64(const double *h, const double *hu,
                                                       const double *hv, int i0, int i1, int Ny,
                                                       long long P, double g,
                                                       unsigned long long *slot) {
    double v = 0.0;
    for (int i = i0 + (int)blockIdx.y; i < i1; i += gridDim.y) {
        const long long r = (long long)(i + NG) * P + NG;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < Ny; j += gridDim.x * blockDim.x)
            v = dmax(v, cell_speed(g, h[r + j], hu[r + j], hv[r + j]));
    }
    block_max_to_slot(v, slot);
}

// Ghost refresh over the perimeter, reproducing apply_reflecting_bc's two sweeps
// (HPC_solver.hpp:326-370): x-ghost rows take the mirrored row (hu negated), y-ghost
// columns over all rows take the mirrored column (hv negated), so a corner holds the
// doubly mirrored interior cell.  Transmissive walls copy the nearest interior cell.
__global__ void k_fill_ghosts_f64(double *h, double *hu, double *hv, int Nx, int Ny,
                                  long long P, int bc, int halo_lo, int halo_hi) {
    const int NyT = Ny + 2 * NG;
    const int n_rows = 4 * NyT;  // rows 0, 1, Nx+2, Nx+3, every column
    const int n_cols = 4 * Nx;   // columns 0, 1, Ny+2, Ny+3 of interior rows
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_rows + n_cols) return;
    int i, j;
    if (t < n_rows) {
        const int r = t / NyT;
        if (r < 2 ? halo_lo : halo_hi) return;  // the neighbour slab's rows
        j = t - r * NyT;
        i = r < 2 ? r : Nx + r;  // 0, 1, Nx+2, Nx+3
    } else {
        const int u = t - n_rows;
        const int c = u / Nx;
        i = NG + (u - c * Nx);
        j = c < 2 ? c : Ny + c;
    }
    bool fx, fy;
    const int si = map_coord(i - NG, Nx, bc, fx) + NG;
    const int sj = map_coord(j - NG, Ny, bc, fy) + NG;
    const long long kd = (long long)i * P + j, ks = (long long)si * P + sj;
    h[kd] = h[ks];
    hu[kd] = fx ? -hu[ks] : hu[ks];
    hv[kd] = fy ? -hv[ks] : hv[ks];
}

// The same ghost rule over ghosted rows [r0, r1) only: whole rows where they are x-ghost
// rows, the four y-ghost columns elsewhere.  Every source cell lies in rows below r1 or
// in the band itself, so a band can be filled (and copied out) as soon as the stage that
// writes its interior rows and those before them has run.
__global__ void k_fill_ghost_band_f64(double *h, double *hu, double *hv, int Nx, int Ny,
                                      long long P, int bc, int r0, int r1) {
    const int NyT = Ny + 2 * NG;
    const int lo = min(max(r0, 0), NG), hi = max(min(r1, Nx + 2 * NG), Nx + NG);
    const int n_lo = max(min(r1, NG) - r0, 0);             // rows 0, 1 in the band
    const int n_hi = max(hi - max(r0, Nx + NG), 0);        // rows Nx+2, Nx+3 in the band
    const int a = max(r0, NG), b = min(r1, Nx + NG);
    const int n_in = max(b - a, 0);                        // interior rows in the band
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int i, j;
    if (t < n_lo * NyT) {
        i = lo + t / NyT;
        j = t - (t / NyT) * NyT;
    } else if (t < (n_lo + n_hi) * NyT) {
        const int u = t - n_lo * NyT;
        i = max(r0, Nx + NG) + u / NyT;
        j = u - (u / NyT) * NyT;
    } else if (t < (n_lo + n_hi) * NyT + 4 * n_in) {
        const int u = t - (n_lo + n_hi) * NyT;
        i = a + (u >> 2);
        const int c = u & 3;
        j = c < 2 ? c : Ny + c;
    } else {
        return;
    }
    bool fx, fy;
    const int si = map_coord(i - NG, Nx, bc, fx) + NG;
    const int sj = map_coord(j - NG, Ny, bc, fy) + NG;
    const long long kd = (long long)i * P + j, ks = (long long)si * P + sj;
    h[kd] = h[ks];
    hu[kd] = fx ? -hu[ks] : hu[ks];
    hv[kd] = fy ? -hv[ks] : hv[ks];
}

}  // namespace

// Once per kernel and device: the largest shared-memory carveout (four tiles of up to
// 47 KB per SM) and, above 48 KB, the opt-in to that much dynamic shared memory.
// `done` is the caller's per-kernel, per-device flag array.
template <class K>
static cudaError_t smem_opt_in(K kernel, size_t bytes, bool (&done)[64]) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e == cudaSuccess && bytes > 48 * 1024)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    done[dev] = true;
    return cudaSuccess;
}

// The strip length for a grid of tiles_j x tile_rows tiles (see SWE_F64_STRIP): the
// whole grid decides, so that the bands of swe_step_host use the length of the grid.
static int strip_tiles_f64(int tiles_j, int tile_rows) {
    if (SWE_F64_STRIP > 0) return SWE_F64_STRIP;
    static int sms[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) !=
                         cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    const long long waves16 = 16LL * min_blocks(8, 32) * sms[dev];
    for (int len : {6, 4})
        if ((long long)tiles_j * ((tile_rows + len - 1) / len) >= waves16) return len;
    return 1;
}

template <int TI, int TJ, int STAGE>
static cudaError_t single_launch_f64(StageParams p, const StageMaps *maps, cudaStream_t s,
                                     int tr0, int tr1) {
    constexpr int NT = (TI + 1) * TJ;
    constexpr size_t smem = sizeof(TileF64<TI, TJ>) + 128;  // + alignment slack
    static bool done[64];  // one per kernel instantiation
    const cudaError_t e = smem_opt_in(k_stage_f64<TI, TJ, STAGE>, smem, done);
    if (e != cudaSuccess) return e;
    const int rows = (p.Nx + TI - 1) / TI;
    if (tr1 < 0 || tr1 > rows) tr1 = rows;
    if (tr0 < 0 || tr0 >= tr1) return tr0 == tr1 ? cudaSuccess : cudaErrorInvalidValue;
    p.tile_row0 = tr0;
    const int strip = strip_tiles_f64((p.Ny + TJ - 1) / TJ, rows);
    const dim3 grid((p.Ny + TJ - 1) / TJ, (tr1 - tr0 + strip - 1) / strip);
    static const StageMaps none{};  // unused when use_tma is 0
    const StageMaps &m = maps ? *maps : none;
    k_stage_f64<TI, TJ, STAGE><<<grid, NT, smem, s>>>(p, m.e, m.u, m.v, m.b, maps ? 1 : 0, tr1,
                                                      strip);
    return cudaGetLastError();
}

cudaError_t launch_stage_f64(int stage, const StageParams &p, const StageMaps *maps,
                             cudaStream_t s, int tile_row0, int tile_row1) {
    static_assert(TILE_I_F64 == 8 && TILE_J_F64 == 32, "tile of the TMA maps");
    switch (stage) {
        case 0: return single_launch_f64<8, 32, 0>(p, maps, s, tile_row0, tile_row1);
        case 1: return single_launch_f64<8, 32, 1>(p, maps, s, tile_row0, tile_row1);
        case 2: return single_launch_f64<8, 32, 2>(p, maps, s, tile_row0, tile_row1);
        default: return single_launch_f64<8, 32, 3>(p, maps, s, tile_row0, tile_row1);
    }
}

// A grid over (column blocks, rows) of at most 8 CTAs per SM: columns by threads, rows
// by CTAs, no per-element division.
static dim3 row_grid(int rows, int cols, int num_sms) {
    const int cap = std::max(num_sms, 1) * 8;
    const int gx = std::max(1, std::min((cols + 255) / 256, cap));
    const int gy = std::max(1, std::min(rows, cap / gx));
    return dim3(gx, gy);
}

cudaError_t launch_combine1_f64(const StageParams &p, void *h, void *hu, void *hv, int num_sms,
                                cudaStream_t s) {
    k_combine1_f64<<<row_grid(p.Nx, p.Ny, num_sms), 256, 0, s>>>(p, static_cast<double *>(h),
                                                      static_cast<double *>(hu),
                                                      static_cast<double *>(hv));
    return cudaGetLastError();
}

template <int TI, int TJ, int STAGE>
static cudaError_t ens_launch_stage(const EnsParams &e, int grid, cudaStream_t s) {
    constexpr int NT = (TI + 1) * TJ;
    constexpr size_t smem = sizeof(TileF64<TI, TJ>) + 128;  // + alignment slack
    static bool done[64];  // one per kernel instantiation
    const cudaError_t err = smem_opt_in(k_ens_stage_f64<TI, TJ, STAGE>, smem, done);
    if (err != cudaSuccess) return err;
    k_ens_stage_f64<TI, TJ, STAGE><<<grid, NT, smem, s>>>(e);
    return cudaGetLastError();
}

template <int TI, int TJ>
static cudaError_t ens_launch_f64(int stage, const EnsParams &e, int grid, cudaStream_t s) {
    switch (stage) {
        case 1: return ens_launch_stage<TI, TJ, 1>(e, grid, s);
        case 2: return ens_launch_stage<TI, TJ, 2>(e, grid, s);
        default: return ens_launch_stage<TI, TJ, 3>(e, grid, s);
    }
}

template <int TI, int TJ, int STAGE>
static int ens_resident_stage_f64() {
    constexpr int NT = (TI + 1) * TJ;
    constexpr size_t smem = sizeof(TileF64<TI, TJ>) + 128;
    static bool done[64];
    if (smem_opt_in(k_ens_stage_f64<TI, TJ, STAGE>, smem, done) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_ens_stage_f64<TI, TJ, STAGE>, NT,
                                                      smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

template <int TI, int TJ>
static int ens_resident_f64() {
    return std::min(ens_resident_stage_f64<TI, TJ, 1>(),
                    std::min(ens_resident_stage_f64<TI, TJ, 2>(), ens_resident_stage_f64<TI, TJ, 3>()));
}

template <int STAGE>
static cudaError_t ens_launch_strip_stage(const EnsParams &e, int grid, cudaStream_t s) {
    constexpr size_t smem = sizeof(TileF64<8, 32>) + 128;
    static bool done[64];
    const cudaError_t err = smem_opt_in(k_ens_stage_f64_strip<STAGE>, smem, done);
    if (err != cudaSuccess) return err;
    k_ens_stage_f64_strip<STAGE><<<grid, 9 * 32, smem, s>>>(e);
    return cudaGetLastError();
}

template <int STAGE>
static int ens_resident_strip_stage() {
    constexpr size_t smem = sizeof(TileF64<8, 32>) + 128;
    static bool done[64];
    if (smem_opt_in(k_ens_stage_f64_strip<STAGE>, smem, done) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_ens_stage_f64_strip<STAGE>, 9 * 32,
                                                      smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int ens_resident_per_sm_f64(int shape) {
    switch (shape) {
        case SHAPE_STRIP:
            return std::min(ens_resident_strip_stage<1>(),
                            std::min(ens_resident_strip_stage<2>(), ens_resident_strip_stage<3>()));
        case SHAPE_8x32: return ens_resident_f64<8, 32>();
        case SHAPE_8x16: return ens_resident_f64<8, 16>();
        case SHAPE_4x64: return ens_resident_f64<4, 64>();
        default: return 0;
    }
}

cudaError_t launch_ens_stage_f64(int shape, int stage, const EnsParams &e, int grid,
                                 cudaStream_t s) {
    switch (shape) {
        case SHAPE_STRIP:
            return stage == 1 ? ens_launch_strip_stage<1>(e, grid, s)
                              : (stage == 2 ? ens_launch_strip_stage<2>(e, grid, s)
                                            : ens_launch_strip_stage<3>(e, grid, s));
        case SHAPE_8x32: return ens_launch_f64<8, 32>(stage, e, grid, s);
        case SHAPE_8x16: return ens_launch_f64<8, 16>(stage, e, grid, s);
        case SHAPE_4x64: return ens_launch_f64<4, 64>(stage, e, grid, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_max_speed_rows_f64(const void *h, const void *hu, const void *hv, int i0,
                                      int i1, int Ny, long long pitch, double g,
                                      unsigned long long *slot, int num_sms, cudaStream_t s) {
    if (i1 <= i0) return cudaSuccess;
    k_max_speed_f64<<<row_grid(i1 - i0, Ny, num_sms), 256, 0, s>>>(
        static_cast<const double *>(h), static_cast<const double *>(hu),
        static_cast<const double *>(hv), i0, i1, Ny, pitch, g, slot);
    return cudaGetLastError();
}

cudaError_t launch_max_speed_f64(const void *h, const void *hu, const void *hv, int Nx, int Ny,
                                 long long pitch, double g, unsigned long long *slot,
                                 int num_sms, cudaStream_t s) {
    return launch_max_speed_rows_f64(h, hu, hv, 0, Nx, Ny, pitch, g, slot, num_sms, s);
}

cudaError_t launch_fill_ghosts_f64(void *h, void *hu, void *hv, int Nx, int Ny, long long pitch,
                                   int bc, cudaStream_t s, int halo_lo, int halo_hi) {
    const int n = 4 * (Ny + 2 * NG) + 4 * Nx;
    k_fill_ghosts_f64<<<(n + 255) / 256, 256, 0, s>>>(static_cast<double *>(h),
                                                       static_cast<double *>(hu),
                                                       static_cast<double *>(hv), Nx, Ny, pitch,
                                                       bc, halo_lo, halo_hi);
    return cudaGetLastError();
}

cudaError_t launch_fill_ghost_band_f64(void *h, void *hu, void *hv, int Nx, int Ny,
                                       long long pitch, int bc, int r0, int r1,
                                       cudaStream_t s) {
    const int NyT = Ny + 2 * NG;
    const int n_lo = std::max(std::min(r1, NG) - r0, 0);
    const int n_hi = std::max(std::min(r1, Nx + 2 * NG) - std::max(r0, Nx + NG), 0);
    const int n_in = std::max(std::min(r1, Nx + NG) - std::max(r0, NG), 0);
    const long long n = (long long)(n_lo + n_hi) * NyT + 4ll * n_in;
    if (n <= 0) return cudaSuccess;
    k_fill_ghost_band_f64<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        static_cast<double *>(h), static_cast<double *>(hu), static_cast<double *>(hv), Nx, Ny,
        pitch, bc, r0, r1);
    return cudaGetLastError();
}

}  // namespace swe
