// FP32-mixed form of the fused SSP-RK3 stage kernel.
//
// Same scheme as the FP64 drop-in (MUSCL on eta, hu, hv; hydrostatic reconstruction
// with b* = max(b-, b+); HLL; SSP-RK3; positivity; walls; CFL reduction), with three
// changes that make FP32 arithmetic safe:
//
//  * The stored state is (eta, hu, hv) with eta = h + B, not (h, hu, hv).  A lake at
//    rest then has a bitwise-constant eta, the MUSCL slopes are exactly zero, and the
//    interface depths eta - b are differences of two FP32 numbers that are exact
//    (Sterbenz) wherever the water is shallow compared with b - the near-dry cells where
//    the reference relies on FP64.
//  * The HLL flux is evaluated as F* = F_L + D with
//    D = s_L (s_R dU - dF) / (s_R - s_L) (or 0 / F_R - F_L in the supersonic cases), and
//    the pressure of the interface depth hs, which the reference adds in the flux and
//    removes in its hydrostatic correction (HPC_kernels.hpp:61-65, 174-183), is dropped
//    from both: the momentum flux seen by the cell on side s is
//    q_n u_n + D_n + g/2 h_s^2.  For equal left/right states D is exactly 0, so the
//    wall pressures of a lake at rest cancel bitwise and hu = hv stay exactly 0.
//  * Time and the CFL dt are FP64 (dt is reduced in FP32, divided in FP64, applied as
//    the FP32 value whose FP64 image is accumulated).
//
// Layout: eta, hu, hv, B are FP32 ghosted arrays with the same pitch rule as the FP64
// form.  The wall boundary condition is applied by mirrored indices while loading.
//
// Kernels: the single grid runs column sweeps (k_stage_f32_cols: a warp marches 28
// columns down a strip of rows with a register window).  Ensembles run the same sweeps
// over work items of 64 x 112 cells (SHAPE_COLS), or tile kernels (8x32, 16x32, 8x64
// tiles staged in shared memory, interior tiles by TMA); the autotuner picks.  Every
// kernel evaluates the interfaces and cell updates with the same explicitly rounded
// arithmetic, so all of them give the same bits.
#include "swe_common.cuh"
#include "swe_launch.h"
#include "swe_tma.cuh"

#include <algorithm>
#include <cstring>

namespace swe {
namespace {

constexpr float EPSF = 1.0e-8f;
constexpr float H_FLOORF = 1.0e-8f;

// Approximate reciprocal and square root (PTX rcp.approx / sqrt.approx, about 1 ulp);
// their error is far below the form's stated L1 budget.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// minmod(a, b) = median(a, b, 0): three min/max, no branches.
__device__ __forceinline__ float minmodf(float a, float b) {
    return fmaxf(fminf(a, b), fminf(fmaxf(a, b), 0.f));
}

struct FaceF {
    float fh, fqt, fqn_m, fqn_p;
};

// The FP32 arithmetic below is written with explicit roundings (__fadd_rn, __fmul_rn,
// fmaf): which products the compiler would fuse depends on the code around an inlined
// copy, and every kernel that evaluates an interface or a cell update (the tile kernels,
// the column sweeps, the ensemble forms) must give the same bits.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// One interface from the 4-cell stencil (m1, c0 | p1, p2) of eta, qn (normal momentum),
// qt (tangential momentum) and the bathymetry of the two adjacent cells.
__device__ __forceinline__ FaceF face_flux_f32(float g, float half_g, float e_m1, float e_0,
                                               float e_p1, float e_p2, float n_m1, float n_0,
                                               float n_p1, float n_p2, float t_m1, float t_0,
                                               float t_p1, float t_p2, float b_m, float b_p) {
    const float eta_m = fmaf(0.5f, minmodf(fsub(e_0, e_m1), fsub(e_p1, e_0)), e_0);
    const float eta_p = fmaf(-0.5f, minmodf(fsub(e_p1, e_0), fsub(e_p2, e_p1)), e_p1);
    const float qn_m = fmaf(0.5f, minmodf(fsub(n_0, n_m1), fsub(n_p1, n_0)), n_0);
    const float qt_m = fmaf(0.5f, minmodf(fsub(t_0, t_m1), fsub(t_p1, t_0)), t_0);
    const float qn_p = fmaf(-0.5f, minmodf(fsub(n_p1, n_0), fsub(n_p2, n_p1)), n_p1);
    const float qt_p = fmaf(-0.5f, minmodf(fsub(t_p1, t_0), fsub(t_p2, t_p1)), t_p1);
    const float b_star = fmaxf(b_m, b_p);
    const float h_m = fmaxf(fsub(eta_m, b_m), 0.f);
    const float h_p = fmaxf(fsub(eta_p, b_p), 0.f);
    const float hs_m = fmaxf(fsub(eta_m, b_star), 0.f);
    const float hs_p = fmaxf(fsub(eta_p, b_star), 0.f);
    const float ih_m = h_m > EPSF ? rcp_approx(h_m) : 0.f;
    const float ih_p = h_p > EPSF ? rcp_approx(h_p) : 0.f;
    const float un_m = fmul(qn_m, ih_m), ut_m = fmul(qt_m, ih_m);
    const float un_p = fmul(qn_p, ih_p), ut_p = fmul(qt_p, ih_p);
    // left / right hydrostatic states and their advective fluxes
    const float qnL = fmul(hs_m, un_m), qtL = fmul(hs_m, ut_m);
    const float qnR = fmul(hs_p, un_p), qtR = fmul(hs_p, ut_p);
    const float aLn = fmul(qnL, un_m), aLt = fmul(qnL, ut_m);
    const float aRn = fmul(qnR, un_p), aRt = fmul(qnR, ut_p);
    const float cL = sqrt_approx(fmul(g, hs_m)), cR = sqrt_approx(fmul(g, hs_p));
    // HLL with the wave speeds clamped to sL- = min(sL, 0), sR+ = max(sR, 0) covers the
    // three regimes without branches: sL >= 0 gives D = 0 (F* = F_L), sR <= 0 gives
    // D = dF (F* = F_R).  At a mirrored wall sL = -sR and k is exactly -1/2, so the wall
    // mass flux cancels exactly.
    const float sLm = fminf(fminf(fsub(un_m, cL), fsub(un_p, cR)), 0.f);
    const float sRp = fmaxf(fmaxf(fadd(un_m, cL), fadd(un_p, cR)), 0.f);
    const float den = fsub(sRp, sLm);
    const float k = (fadd(sLm, sRp) == 0.f) ? (den > 0.f ? -0.5f : 0.f)
                                           : fmul(sLm, rcp_approx(fmaxf(den, 1e-30f)));
    const float dhs = fsub(hs_p, hs_m);
    const float dFh = fsub(qnR, qnL);
    const float dFn = fmaf(fmul(half_g, dhs), fadd(hs_p, hs_m), fsub(aRn, aLn));
    const float dFt = fsub(aRt, aLt);
    // F* = F_L + D with D = k (s_R+ dU - dF), each fused into one rounding: F* is often
    // much smaller than F_L and D, and a rounded product would leave an error of the size
    // of F_L in it.
    // fqn_m = F*_n + g/2 (h_m^2 - hs_m^2) = aLn + Dn + g/2 h_m^2
    // fqn_p = F*_n + g/2 (h_p^2 - hs_p^2) = aLn + Dn + g/2 (hs_m^2 - hs_p^2) + g/2 h_p^2
    FaceF f;
    f.fh = fmaf(k, fmaf(sRp, dhs, -dFh), qnL);
    f.fqt = fmaf(k, fmaf(sRp, fsub(qtR, qtL), -dFt), aLt);
    const float base = fmaf(k, fmaf(sRp, fsub(qnR, qnL), -dFn), aLn);
    f.fqn_m = fmaf(fmul(half_g, h_m), h_m, base);
    f.fqn_p = fmaf(fmul(half_g, h_p), h_p,
                   fmaf(fmul(half_g, fsub(hs_m, hs_p)), fadd(hs_m, hs_p), base));
    return f;
}

__device__ __forceinline__ float cell_speed_f32(float g, float h, float hu, float hv) {
    const float ih = h > EPSF ? rcp_approx(h) : 0.f;
    const float c = sqrt_approx(fmul(g, fmaxf(h, 0.f)));
    return fmaxf(fadd(fabsf(fmul(hu, ih)), c), fadd(fabsf(fmul(hv, ih)), c));
}

// A ghost cell's eta: the source cell's depth over the ghost's own bed (eta itself where
// the beds agree, so a flat surface stays bitwise flat).
__device__ __forceinline__ float ghost_eta(float e, float bsrc, float b) {
    return (b == bsrc) ? e : fadd(fsub(e, bsrc), b);
}

// The flux divergence of one cell from its four interfaces (apply_divergence's
// -inv_dx (right - left) - inv_dy (top - bottom)).
__device__ __forceinline__ float divergence(float idx, float idy, float xhi, float xlo,
                                            float yhi, float ylo) {
    return fmaf(-idy, fsub(yhi, ylo), fmul(-idx, fsub(xhi, xlo)));
}

// Stage combine of one field: 1: s + dt L; 2: 3/4 n + 1/4 (s + dt L); 3: n + c (s' - n)
// with c = fl(2/3), s' = s + dt L (the FP32 weights fl(1/3) + fl(2/3) exceed 1 by 3e-8,
// which would add mass every step; these sum to 1).
template <int STAGE>
__device__ __forceinline__ float combine_f32(float s, float n, float dt, float L) {
    const float e = fmaf(dt, L, s);
    if (STAGE == 1) return e;
    if (STAGE == 2) return fmaf(0.75f, n, fmul(0.25f, e));
    return fmaf(2.f / 3.f, fsub(e, n), n);
}

__device__ __forceinline__ void block_max_to_slot_f(float v, unsigned long long *slot) {
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? red[lane] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.f)
            atomicMax(slot, (unsigned long long)__double_as_longlong((double)v));
    }
}

// The step's dt, computed once per block in FP64 and shared together with its FP32
// image (an FP64 division or conversion per thread runs on GB300's slow FP64 unit).
struct BlockDt {
    double d;
    float f;
};

// The block's dt; `abort` is true (block-uniform) when FLAG_TIMEOUT is already set, read
// under the same barrier.
__device__ __forceinline__ BlockDt stage_dt_f32(const StageParams &p, bool &abort) {
    __shared__ double s_dt;
    __shared__ float s_dtf;
    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        double dt = p.dt_fixed;
        if (!(dt > 0.0)) {
            const double ms = __longlong_as_double((long long)p.speed[p.slot_read]);
            dt = (ms <= EPS) ? 1.0e100 : p.cfl_min_dxdy / ms;
        }
        s_dt = dt;
        s_dtf = (float)dt;
        s_abort = tma::timeout_set(p.flags);
    }
    __syncthreads();
    abort = s_abort != 0;
    return BlockDt{s_dt, s_dtf};
}

// One tile of one RK stage (see stage_tile_f64); returns the thread's cell wave speed of
// the new state in stage 3, else 0.  (TI + 1) * TJ threads; dt is the block's dt.
// Interior tiles are staged by TMA through `pipe` when tm is given; `aborted` is set
// (block-uniform) when that wait gave up, and the caller then returns from the kernel.
template <int TI, int TJ, int STAGE>
__device__ __forceinline__ float stage_tile_f32(const StageParams &p, int i0, int j0,
                                                float dt, const tma::TileMaps *tm,
                                                tma::Pipe &pipe, bool &aborted) {
    constexpr int NT = (TI + 1) * TJ, RI = TI + 4, RJ = TJ + 4;
    // 128-byte aligned so the TMA box of each field lands on an aligned address
    __shared__ __align__(128) float s_e[RI][RJ];
    __shared__ __align__(128) float s_u[RI][RJ];
    __shared__ __align__(128) float s_v[RI][RJ];
    __shared__ __align__(128) float s_b[RI][RJ];
    __shared__ float s_xf[4][TI + 1][TJ];
    __shared__ float s_yf[4][TI][TJ + 1];

    const int tid = threadIdx.x;
    const long long P = p.pitch;
    const float *es = static_cast<const float *>(p.hs);
    const float *us = static_cast<const float *>(p.hus);
    const float *vs = static_cast<const float *>(p.hvs);
    const float *Bg = static_cast<const float *>(p.B);

    // Tiles whose halo lies inside the interior are staged by TMA; tiles that touch a
    // wall use mirrored indices (their halo holds ghost cells).
    const bool interior = tm != nullptr && i0 >= NG && j0 >= NG && i0 + TI + NG <= p.Nx &&
                          j0 + TJ + NG <= p.Ny;
    aborted = false;
    if (interior) {
        // halo origin (i0 - 2, j0 - 2) in interior coordinates = (i0, j0) in the ghosted
        // array; j0 is a multiple of TJ, so x * 4 bytes is 16-byte aligned
        uint64_t *bar = pipe.bar;
        if (!tma::stage_in(pipe, p.flags, 4u * RI * RJ * sizeof(float), [&] {
                tma::load_2d(&s_e[0][0], tm->e, j0, i0, bar);
                tma::load_2d(&s_u[0][0], tm->u, j0, i0, bar);
                tma::load_2d(&s_v[0][0], tm->v, j0, i0, bar);
                tma::load_2d(&s_b[0][0], tm->b, j0, i0, bar);
            })) {
            aborted = true;
            return 0.f;
        }
    } else {
        for (int t = tid; t < RI * RJ; t += NT) {
            const int r = t / RJ, c = t - (t / RJ) * RJ;
            const int ii = i0 - NG + r, jj = j0 - NG + c;
            bool fx, fy;
            const int mi = map_coord(ii, p.Nx, p.bc, fx);
            const int mj = map_coord(jj, p.Ny, p.bc, fy);
            const long long k = (long long)(mi + NG) * P + (mj + NG);
            const int bi = clamp_int(ii + NG, 0, p.Nx + 2 * NG - 1);
            const int bj = clamp_int(jj + NG, 0, p.Ny + 2 * NG - 1);
            const float b = Bg[(long long)bi * P + bj];
            // A ghost holds the interior cell's depth over its own bed: eta_g = h_src + B_g
            // (eta itself where the beds agree, so a flat surface stays bitwise flat).
            s_e[r][c] = ghost_eta(es[k], Bg[k], b);
            const float u = us[k], v = vs[k];
            s_u[r][c] = fx ? -u : u;
            s_v[r][c] = fy ? -v : v;
            s_b[r][c] = b;
        }
        __syncthreads();
    }

    const float g = p.gf, half_g = p.half_gf;
    {
        const int fr = tid / TJ, fc = tid - (tid / TJ) * TJ;
        const int a = fr + 1, c = fc + NG;
        const FaceF F = face_flux_f32(g, half_g, s_e[a - 1][c], s_e[a][c], s_e[a + 1][c],
                                      s_e[a + 2][c], s_u[a - 1][c], s_u[a][c], s_u[a + 1][c],
                                      s_u[a + 2][c], s_v[a - 1][c], s_v[a][c], s_v[a + 1][c],
                                      s_v[a + 2][c], s_b[a][c], s_b[a + 1][c]);
        s_xf[0][fr][fc] = F.fh;
        s_xf[1][fr][fc] = F.fqt;
        s_xf[2][fr][fc] = F.fqn_m;
        s_xf[3][fr][fc] = F.fqn_p;
    }
    if (tid < TI * (TJ + 1)) {
        const int fr = tid / (TJ + 1), fc = tid - (tid / (TJ + 1)) * (TJ + 1);
        const int r = fr + NG, a = fc + 1;
        const FaceF F = face_flux_f32(g, half_g, s_e[r][a - 1], s_e[r][a], s_e[r][a + 1],
                                      s_e[r][a + 2], s_v[r][a - 1], s_v[r][a], s_v[r][a + 1],
                                      s_v[r][a + 2], s_u[r][a - 1], s_u[r][a], s_u[r][a + 1],
                                      s_u[r][a + 2], s_b[r][a], s_b[r][a + 1]);
        s_yf[0][fr][fc] = F.fh;
        s_yf[1][fr][fc] = F.fqt;
        s_yf[2][fr][fc] = F.fqn_m;
        s_yf[3][fr][fc] = F.fqn_p;
    }
    __syncthreads();

    const int ty = tid / TJ, tx = tid - (tid / TJ) * TJ;
    const int ii = i0 + ty, jj = j0 + tx;
    const bool inside = (ty < TI) && (ii < p.Nx) && (jj < p.Ny);
    float speed = 0.f;
    if (inside) {
        const float idx = p.inv_dxf, idy = p.inv_dyf;
        const float rh = divergence(idx, idy, s_xf[0][ty + 1][tx], s_xf[0][ty][tx],
                                    s_yf[0][ty][tx + 1], s_yf[0][ty][tx]);
        const float rhu = divergence(idx, idy, s_xf[2][ty + 1][tx], s_xf[3][ty][tx],
                                     s_yf[1][ty][tx + 1], s_yf[1][ty][tx]);
        const float rhv = divergence(idx, idy, s_xf[1][ty + 1][tx], s_xf[1][ty][tx],
                                     s_yf[2][ty][tx + 1], s_yf[3][ty][tx]);
        const long long k = (long long)(ii + NG) * P + (jj + NG);
        const float se = s_e[ty + NG][tx + NG], su = s_u[ty + NG][tx + NG];
        const float sv = s_v[ty + NG][tx + NG], b = s_b[ty + NG][tx + NG];
        float ne = 0.f, nu = 0.f, nv = 0.f;
        if (STAGE != 1) {
            ne = static_cast<const float *>(p.hn)[k];
            nu = static_cast<const float *>(p.hun)[k];
            nv = static_cast<const float *>(p.hvn)[k];
        }
        float oe = combine_f32<STAGE>(se, ne, dt, rh);
        float ou = combine_f32<STAGE>(su, nu, dt, rhu);
        float ov = combine_f32<STAGE>(sv, nv, dt, rhv);
        const bool clamped = fsub(oe, b) < H_FLOORF;
        if (clamped) {  // enforce_positivity on h = eta - B
            oe = fadd(b, H_FLOORF);
            ou = 0.f;
            ov = 0.f;
        }
        if (p.mask) p.mask[k] = clamped ? 1 : 0;  // for the adjoint
        if (!(fabsf(oe) + fabsf(ou) + fabsf(ov) < INFINITY)) atomicOr(p.flags, FLAG_NONFINITE);
        static_cast<float *>(p.ho)[k] = oe;
        static_cast<float *>(p.huo)[k] = ou;
        static_cast<float *>(p.hvo)[k] = ov;
        if (STAGE == 3) speed = cell_speed_f32(g, fsub(oe, b), ou, ov);
    }
    return speed;
}

// ---- Single grid: column sweeps --------------------------------------------------------
//
// Each warp owns 28 consecutive columns and one strip of F32_STRIP rows.  Lane l holds
// column 28 g - 2 + l (lanes 0-1 and 30-31 are the neighbours' columns, the stencil
// halo) and marches down the rows with a window of four rows of (eta, hu, hv, B) in
// registers, loading each row once, straight from global memory: no shared-memory tile,
// no barrier per tile.  At row r it computes the x-interface between rows r and r + 1
// from its own window (the interface between r - 1 and r is the previous row's), and
// the y-interface between its column and the next from row r of lanes l - 1 .. l + 2
// (warp shuffles); the y-interface on its other side is lane l - 1's.  Lanes 2-29 then
// update their cell.  Ghost cells are loaded through the same mirrored or clamped indices
// as the tile loader, so every interface sees the values the tile kernel sees and the
// arithmetic (face_flux_f32, the cell update) is the same.
#ifndef SWE_F32_STRIP
#define SWE_F32_STRIP F32_STRIP_ROWS
#endif
constexpr int F32_COLS = 28, F32_WARPS = 4;
static_assert(F32_COLS * F32_WARPS == F32_COL_BLOCK, "SHAPE_COLS work item width");

struct RowF {
    float e, u, v, b;
};

// Where the column sweep finds a grid's fields and constants.  GridAcc: one context's
// stage, all in the kernel's parameters (constant bank).  EnsAcc: one ensemble
// instance, its fields at a byte offset from the ensemble's pools (parameters) and its
// sizes in registers.
struct GridAcc {
    const StageParams &p;
    __device__ int Nx() const { return p.Nx; }
    __device__ int Ny() const { return p.Ny; }
    __device__ long long pitch() const { return p.pitch; }
    __device__ int bc() const { return p.bc; }
    __device__ float idx() const { return p.inv_dxf; }
    __device__ float idy() const { return p.inv_dyf; }
    __device__ float g() const { return p.gf; }
    __device__ float half_g() const { return p.half_gf; }
    __device__ const float *src(int f) const {
        return static_cast<const float *>(f == 0 ? p.hs : (f == 1 ? p.hus : p.hvs));
    }
    __device__ const float *n(int f) const {
        return static_cast<const float *>(f == 0 ? p.hn : (f == 1 ? p.hun : p.hvn));
    }
    __device__ float *out(int f) const {
        return static_cast<float *>(f == 0 ? p.ho : (f == 1 ? p.huo : p.hvo));
    }
    __device__ const float *B() const { return static_cast<const float *>(p.B); }
    __device__ unsigned char *mask() const { return p.mask; }
    __device__ int *flags() const { return p.flags; }
};

struct EnsAcc {
    const EnsParams &e;
    long long off;  // bytes
    int nx, ny;
    long long pt;
    float ix, iy;
    __device__ int Nx() const { return nx; }
    __device__ int Ny() const { return ny; }
    __device__ long long pitch() const { return pt; }
    __device__ int bc() const { return e.bc; }
    __device__ float idx() const { return ix; }
    __device__ float idy() const { return iy; }
    __device__ float g() const { return e.gf; }
    __device__ float half_g() const { return e.half_gf; }
    __device__ const float *src(int f) const {
        return reinterpret_cast<const float *>(static_cast<const char *>(e.src[f]) + off);
    }
    __device__ const float *n(int f) const {
        return reinterpret_cast<const float *>(static_cast<const char *>(e.n[f]) + off);
    }
    __device__ float *out(int f) const {
        return reinterpret_cast<float *>(static_cast<char *>(e.out[f]) + off);
    }
    __device__ const float *B() const {
        return reinterpret_cast<const float *>(static_cast<const char *>(e.B) + off);
    }
    __device__ unsigned char *mask() const { return nullptr; }
    __device__ int *flags() const { return e.flags; }
};

// Row ii (interior coordinates, possibly outside) of lane column jj, as the tile loader
// stages it: ghosts mirror or clamp by the wall rule, B is read where it lies, and a
// ghost's eta is its source cell's depth over the ghost's own bed.
template <class Acc>
__device__ __forceinline__ RowF load_row_f32(const Acc &a, int ii, int mj, bool fy, int bj) {
    bool fx;
    const int mi = map_coord(ii, a.Nx(), a.bc(), fx);
    const int bi = clamp_int(ii + NG, 0, a.Nx() + 2 * NG - 1);
    const long long k = (long long)(mi + NG) * a.pitch() + (mj + NG);
    const long long kb = (long long)bi * a.pitch() + bj;
    const float *Bg = a.B();
    RowF r;
    const float e = a.src(0)[k];
    const float u = a.src(1)[k];
    const float v = a.src(2)[k];
    r.b = Bg[kb];
    r.e = ghost_eta(e, kb == k ? r.b : Bg[k], r.b);
    r.u = fx ? -u : u;
    r.v = fy ? -v : v;
    return r;
}

// One warp's sweep: column group grp (columns 28 grp .. 28 grp + 27), rows [r0, r1) of
// the grid a describes; returns the lane's max wave speed of the new state (stage 3).
template <int STAGE, class Acc>
__device__ __forceinline__ float col_sweep_f32(const Acc &a, int grp, int r0, int r1, float dt) {
    const int lane = threadIdx.x & 31;
    const int jj = grp * F32_COLS - NG + lane;  // this lane's column
    bool fy;
    const int mj = map_coord(jj, a.Ny(), a.bc(), fy);
    const int bj = clamp_int(jj + NG, 0, a.Ny() + 2 * NG - 1);
    const bool out_col = lane >= NG && lane < NG + F32_COLS && jj < a.Ny();
    const float g = a.g(), half_g = a.half_g(), idx = a.idx(), idy = a.idy();
    float speed = 0.f;
    // window: rows r - 1, r, r + 1, r + 2 for the x-interface between r and r + 1
    RowF w0 = load_row_f32(a, r0 - 2, mj, fy, bj), w1 = load_row_f32(a, r0 - 1, mj, fy, bj);
    RowF w2 = load_row_f32(a, r0, mj, fy, bj), w3 = load_row_f32(a, r0 + 1, mj, fy, bj);
    FaceF xlo{};  // the x-interface below row r
    // U^n of the lane's cell in row r (stages 2 and 3), loaded a row ahead; lanes without
    // an output cell read their mapped column, which is inside the grid
    auto load_n = [&](int r, float &ne, float &nu, float &nv) {
        if (STAGE == 1 || r >= r1) return;
        const long long k = (long long)(r + NG) * a.pitch() + (mj + NG);
        ne = a.n(0)[k];
        nu = a.n(1)[k];
        nv = a.n(2)[k];
    };
    float ne = 0.f, nu = 0.f, nv = 0.f;
    load_n(r0, ne, nu, nv);
    for (int r = r0 - 1; r < r1; ++r) {
        const RowF nx = load_row_f32(a, r + 3, mj, fy, bj);  // in flight during the row
        float ne1 = 0.f, nu1 = 0.f, nv1 = 0.f;
        if (r >= r0) load_n(r + 1, ne1, nu1, nv1);
        const FaceF xhi = face_flux_f32(g, half_g, w0.e, w1.e, w2.e, w3.e, w0.u, w1.u, w2.u,
                                        w3.u, w0.v, w1.v, w2.v, w3.v, w1.b, w2.b);
        if (r >= r0) {
            // row r is w1; the y-interface between this column and the next
            const unsigned all = 0xffffffffu;
            const float em1 = __shfl_up_sync(all, w1.e, 1), ep1 = __shfl_down_sync(all, w1.e, 1);
            const float ep2 = __shfl_down_sync(all, w1.e, 2);
            const float vm1 = __shfl_up_sync(all, w1.v, 1), vp1 = __shfl_down_sync(all, w1.v, 1);
            const float vp2 = __shfl_down_sync(all, w1.v, 2);
            const float um1 = __shfl_up_sync(all, w1.u, 1), up1 = __shfl_down_sync(all, w1.u, 1);
            const float up2 = __shfl_down_sync(all, w1.u, 2);
            const float bp1 = __shfl_down_sync(all, w1.b, 1);
            const FaceF yhi = face_flux_f32(g, half_g, em1, w1.e, ep1, ep2, vm1, w1.v, vp1, vp2,
                                            um1, w1.u, up1, up2, w1.b, bp1);
            FaceF ylo;  // the y-interface on the other side is the previous lane's
            ylo.fh = __shfl_up_sync(all, yhi.fh, 1);
            ylo.fqt = __shfl_up_sync(all, yhi.fqt, 1);
            ylo.fqn_m = __shfl_up_sync(all, yhi.fqn_m, 1);
            ylo.fqn_p = __shfl_up_sync(all, yhi.fqn_p, 1);
            if (out_col) {
                const float rh = divergence(idx, idy, xhi.fh, xlo.fh, yhi.fh, ylo.fh);
                const float rhu = divergence(idx, idy, xhi.fqn_m, xlo.fqn_p, yhi.fqt, ylo.fqt);
                const float rhv = divergence(idx, idy, xhi.fqt, xlo.fqt, yhi.fqn_m, ylo.fqn_p);
                const long long k = (long long)(r + NG) * a.pitch() + (jj + NG);
                const float b = w1.b;
                float oe = combine_f32<STAGE>(w1.e, ne, dt, rh);
                float ou = combine_f32<STAGE>(w1.u, nu, dt, rhu);
                float ov = combine_f32<STAGE>(w1.v, nv, dt, rhv);
                const bool clamped = fsub(oe, b) < H_FLOORF;
                if (clamped) {  // enforce_positivity on h = eta - B
                    oe = fadd(b, H_FLOORF);
                    ou = 0.f;
                    ov = 0.f;
                }
                unsigned char *mask = a.mask();
                if (mask) mask[k] = clamped ? 1 : 0;  // for the adjoint
                if (!(fabsf(oe) + fabsf(ou) + fabsf(ov) < INFINITY))
                    atomicOr(a.flags(), FLAG_NONFINITE);
                a.out(0)[k] = oe;
                a.out(1)[k] = ou;
                a.out(2)[k] = ov;
                if (STAGE == 3) speed = fmaxf(speed, cell_speed_f32(g, fsub(oe, b), ou, ov));
            }
        }
        xlo = xhi;
        w0 = w1;
        w1 = w2;
        w2 = w3;
        w3 = nx;
        if (r >= r0) {
            ne = ne1;
            nu = nu1;
            nv = nv1;
        }
    }
    return speed;
}

// Eight 128-thread CTAs per SM (64 registers): stage 3 otherwise takes 71 registers and
// seven CTAs (16384^2 on one box: 22.7 GCUPS uncapped, 24.5 capped, 19.4 at ten CTAs).
#ifndef SWE_F32_COL_MIN_BLOCKS
#define SWE_F32_COL_MIN_BLOCKS 8
#endif
template <int STAGE, int STRIP>
__global__ void __launch_bounds__(32 * F32_WARPS, SWE_F32_COL_MIN_BLOCKS)
    k_stage_f32_cols(const StageParams p) {
    bool aborted;
    const BlockDt bd = stage_dt_f32(p, aborted);
    if (aborted) return;  // an earlier wait of this call gave up
    const float dt = bd.f;
    const int grp = blockIdx.x * F32_WARPS + (threadIdx.x >> 5);
    const int r0 = blockIdx.y * STRIP, r1 = min(r0 + STRIP, p.Nx);
    float speed = 0.f;
    if (grp * F32_COLS < p.Ny) speed = col_sweep_f32<STAGE>(GridAcc{p}, grp, r0, r1, dt);
    if (STAGE == 1 && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        p.speed[p.slot_write] = 0ull;
        if (p.dt_log) p.dt_log[p.log_index] = (double)dt;
    }
    if (STAGE == 3) {
        block_max_to_slot_f(speed, p.speed + p.slot_write);
        if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && p.t_accum)
            *p.t_accum += (double)dt;
    }
}

// Ensemble form of the column sweeps: work item = (instance, block of F32_WARPS column
// groups, strip of SWE_F32_STRIP rows), the SHAPE_COLS tiles of the work list.  The
// schedule is the tile kernel's: one CTA per item, or contiguous shares of the list, with
// the instance's view, dt and first-item duties set up once per instance met.
// Eight 128-thread CTAs per SM (64 registers): the per-instance addresses otherwise take
// the ensemble sweep to 94 registers and 13.8 GCUPS on the 512-instance workload; with
// the cap it runs at 18.6 (6 CTAs: 16.3).
#ifndef SWE_ENS_F32_COL_MIN_BLOCKS
#define SWE_ENS_F32_COL_MIN_BLOCKS 8
#endif
template <int STAGE>
__global__ void __launch_bounds__(32 * F32_WARPS, SWE_ENS_F32_COL_MIN_BLOCKS)
    k_ens_stage_f32_cols(const EnsParams e) {
    __shared__ StageParams s_p;
    __shared__ int s_q, s_t, s_ntiles, s_abort;
    __shared__ float s_dtf;
    const int total = e.total_tiles;
    int T0 = blockIdx.x, T1 = blockIdx.x + 1;
    if ((int)gridDim.x < total) {
        const int per = (total + (int)gridDim.x - 1) / (int)gridDim.x;
        T0 = blockIdx.x * per;
        T1 = min(total, T0 + per);
    }
    for (int T = T0; T < T1; ++T) {
        if (threadIdx.x == 0) {
            int q = s_q, t = s_t + 1;
            const bool fresh = T == T0 || t == s_ntiles;
            if (T == T0) {
                q = e.tile_inst[T];
                t = T - e.inst[q].tile_base;
            } else if (t == s_ntiles) {
                q = q + 1;  // the work list holds the instances' items in instance order
                t = 0;
            }
            if (fresh) {
                s_p = ens_view(e, q);
                s_ntiles = ((e.inst[q].Nx + SWE_F32_STRIP - 1) / SWE_F32_STRIP) * e.inst[q].tiles_j;
                double dt = e.dt_fixed;
                if (!(dt > 0.0)) {
                    const double ms = __longlong_as_double((long long)s_p.speed[s_p.slot_read]);
                    dt = (ms <= EPS) ? 1.0e100 : s_p.cfl_min_dxdy / ms;
                }
                s_dtf = (float)dt;
            }
            s_q = q;
            s_t = t;
            s_abort = tma::timeout_set(e.flags);
        }
        __syncthreads();
        if (s_abort) return;  // the call has failed: the launch ends
        const StageParams &p = s_p;
        const int q = s_q, t = s_t;
        const EnsInst &I = e.inst[q];
        const EnsAcc acc{e, I.off * e.elem, I.Nx, I.Ny, I.pitch, I.inv_dxf, I.inv_dyf};
        const int tiles_j = I.tiles_j;
        const int ti = t / tiles_j, tj = t - (t / tiles_j) * tiles_j;
        const float dt = s_dtf;
        const int grp = tj * F32_WARPS + (threadIdx.x >> 5);
        const int r0 = ti * SWE_F32_STRIP, r1 = min(r0 + SWE_F32_STRIP, acc.nx);
        float speed = 0.f;
        if (grp * F32_COLS < acc.ny) speed = col_sweep_f32<STAGE>(acc, grp, r0, r1, dt);
        if (STAGE == 1 && t == 0 && threadIdx.x == 0) {
            p.speed[p.slot_write] = 0ull;
            if (e.dt_last) e.dt_last[q] = (double)dt;  // the FP32 dt the update applied
        }
        if (STAGE == 3) {
            block_max_to_slot_f(speed, p.speed + p.slot_write);
            if (t == 0 && threadIdx.x == 0) e.t[q] += (double)dt;
        }
        __syncthreads();  // the next item reuses the view
    }
}

#ifndef SWE_ENS_F32_THREADS_PER_SM
#define SWE_ENS_F32_THREADS_PER_SM 2016  // seven 8x32 tiles, the single-grid occupancy
#endif
constexpr int ens_min_blocks_f32(int TI, int TJ) {
    return SWE_ENS_F32_THREADS_PER_SM / ((TI + 1) * TJ) > 0
               ? SWE_ENS_F32_THREADS_PER_SM / ((TI + 1) * TJ) : 1;
}

template <int TI, int TJ, int STAGE>
__global__ void __launch_bounds__((TI + 1) * TJ, ens_min_blocks_f32(TI, TJ))
    k_ens_stage_f32(const EnsParams e) {
    // The instance's view lives in shared memory, read where used, as the single-grid
    // kernel reads its parameters from the constant bank (held in registers it halves
    // the resident CTAs).
    //
    // With fewer CTAs than tiles (a persistent schedule) each CTA takes a contiguous
    // range of the work list, so consecutive tiles mostly belong to one instance: the
    // view, the instance's dt and its TMA maps are set up once per instance the range
    // touches, not once per tile, and the next tile's instance needs no global lookup.
    __shared__ StageParams s_p;
    __shared__ int s_q, s_t, s_ntiles, s_abort;
    __shared__ float s_dtf;
    __shared__ __align__(8) uint64_t s_bar;
    if (e.maps && threadIdx.x == 0) tma::mbar_init(&s_bar, 1);  // visible after the first barrier
    tma::Pipe pipe{&s_bar, 0u};
    const int total = e.total_tiles;
    int T0 = blockIdx.x, T1 = blockIdx.x + 1;
    if ((int)gridDim.x < total) {
        const int per = (total + (int)gridDim.x - 1) / (int)gridDim.x;
        T0 = blockIdx.x * per;
        T1 = min(total, T0 + per);
    }
    for (int T = T0; T < T1; ++T) {
        if (threadIdx.x == 0) {
            int q = s_q, t = s_t + 1;
            const bool fresh = T == T0 || t == s_ntiles;
            if (T == T0) {
                q = e.tile_inst[T];
                t = T - e.inst[q].tile_base;
            } else if (t == s_ntiles) {
                q = q + 1;  // the work list holds the instances' tiles in instance order
                t = 0;
            }
            if (fresh) {
                s_p = ens_view(e, q);
                s_ntiles = ((e.inst[q].Nx + TI - 1) / TI) * e.inst[q].tiles_j;
                // the instance's dt of this step, as stage_dt_f32
                double dt = e.dt_fixed;
                if (!(dt > 0.0)) {
                    const double ms = __longlong_as_double((long long)s_p.speed[s_p.slot_read]);
                    dt = (ms <= EPS) ? 1.0e100 : s_p.cfl_min_dxdy / ms;
                }
                s_dtf = (float)dt;
            }
            s_q = q;
            s_t = t;
            s_abort = tma::timeout_set(e.flags);
        }
        __syncthreads();
        if (s_abort) return;  // a wait of this call gave up: the whole launch ends
        const StageParams &p = s_p;
        const int q = s_q, t = s_t;
        const int tiles_j = e.inst[q].tiles_j;
        const int ti = t / tiles_j, tj = t - (t / tiles_j) * tiles_j;
        const float dt = s_dtf;
        tma::TileMaps tm{};
        if (e.maps) {
            const CUtensorMap *m =
                static_cast<const CUtensorMap *>(e.maps) + ((size_t)q * 3 + (STAGE - 1)) * 4;
            tm = tma::TileMaps{m, m + 1, m + 2, m + 3};
        }
        bool aborted;
        const float speed = stage_tile_f32<TI, TJ, STAGE>(p, ti * TI, tj * TJ, dt,
                                                          e.maps ? &tm : nullptr, pipe, aborted);
        if (aborted) return;
        if (STAGE == 1 && t == 0 && threadIdx.x == 0) {
            p.speed[p.slot_write] = 0ull;
            if (e.dt_last) e.dt_last[q] = (double)dt;  // the FP32 dt the update applied
        }
        if (STAGE == 3) {
            block_max_to_slot_f(speed, p.speed + p.slot_write);
            if (t == 0 && threadIdx.x == 0) e.t[q] += (double)dt;
        }
        __syncthreads();  // the next tile reuses the shared tile buffers and the view
    }
}

__global__ void __launch_bounds__(256) k_max_speed_f32(const float *e, const float *hu,
                                                       const float *hv, const float *B, int Nx,
                                                       int Ny, long long P, float g,
                                                       unsigned long long *slot) {
    float v = 0.f;
    const long long n = (long long)Nx * Ny;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / Ny), j = (int)(t - (t / Ny) * Ny);
        const long long k = (long long)(i + NG) * P + (j + NG);
        v = fmaxf(v, cell_speed_f32(g, e[k] - B[k], hu[k], hv[k]));
    }
    block_max_to_slot_f(v, slot);
}

// FP64 host-layout staging <-> FP32 device state, for all (Nx+4) x (Ny+4) cells.
// to_device: eta = RN32(h + B), hu, hv = RN32; B = RN32(B).
__global__ void k_f64_to_f32(const double *src, const double *add, float *dst, int rows,
                             int cols, long long P) {
    const long long n = (long long)rows * cols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / cols), j = (int)(t - (t / cols) * cols);
        const long long k = (long long)i * P + j;
        const double v = add ? src[k] + add[k] : src[k];
        dst[k] = (float)v;
    }
}

// to_host: h = eta - B (exact in FP64 for FP32 operands), hu, hv widened.
__global__ void k_f32_to_f64(const float *src, const float *sub, double *dst, int rows, int cols,
                             long long P) {
    const long long n = (long long)rows * cols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / cols), j = (int)(t - (t / cols) * cols);
        const long long k = (long long)i * P + j;
        dst[k] = sub ? (double)src[k] - (double)sub[k] : (double)src[k];
    }
}

// Ghost refresh of the FP32 state: as k_fill_ghosts_f64, with the ghost's free surface
// rebuilt over its own bed (eta_g = eta_src - B_src + B_g) so the depth is mirrored.
__global__ void k_fill_ghosts_f32(float *e, float *hu, float *hv, const float *B, int Nx, int Ny,
                                  long long P, int bc) {
    const int NyT = Ny + 2 * NG;
    const int n_rows = 4 * NyT, n_cols = 4 * Nx;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_rows + n_cols) return;
    int i, j;
    if (t < n_rows) {
        const int r = t / NyT;
        j = t - r * NyT;
        i = r < 2 ? r : Nx + r;
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
    e[kd] = (B[kd] == B[ks]) ? e[ks] : (e[ks] - B[ks]) + B[kd];
    hu[kd] = fx ? -hu[ks] : hu[ks];
    hv[kd] = fy ? -hv[ks] : hv[ks];
}

unsigned grid_for(long long n, int num_sms) {
    long long blocks = (n + 255) / 256;
    const long long cap = (long long)num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace

cudaError_t launch_stage_f32(int stage, const StageParams &p, const StageMaps *maps,
                             cudaStream_t s) {
    (void)maps;  // the column sweeps read global memory directly
    const int groups = (p.Ny + F32_COLS - 1) / F32_COLS;
    // Strips of SWE_F32_STRIP rows, shorter on small grids so that there are warps enough
    // to fill the GPU (a strip costs four extra row loads; 1024^2 in strips of 64 rows
    // would be 160 CTAs).
    static_assert(SWE_F32_STRIP == 64, "the strip lengths compiled below");
    int strip = SWE_F32_STRIP;
    const long long kWarps = 8192;
    while (strip > 8 && (long long)groups * ((p.Nx + strip - 1) / strip) < kWarps) strip /= 2;
    const dim3 grid((groups + F32_WARPS - 1) / F32_WARPS, (p.Nx + strip - 1) / strip);
    switch (stage * 1000 + strip) {  // the strip length is a template parameter: a loop
                                     // bound known to the compiler is worth 10% at 16384^2
        case 1064: k_stage_f32_cols<1, 64><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 1032: k_stage_f32_cols<1, 32><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 1016: k_stage_f32_cols<1, 16><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 1008: k_stage_f32_cols<1, 8><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 2064: k_stage_f32_cols<2, 64><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 2032: k_stage_f32_cols<2, 32><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 2016: k_stage_f32_cols<2, 16><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 2008: k_stage_f32_cols<2, 8><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 3064: k_stage_f32_cols<3, 64><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 3032: k_stage_f32_cols<3, 32><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 3016: k_stage_f32_cols<3, 16><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        case 3008: k_stage_f32_cols<3, 8><<<grid, 32 * F32_WARPS, 0, s>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int TI, int TJ>
static cudaError_t ens_launch_f32(int stage, const EnsParams &e, int grid, cudaStream_t s) {
    constexpr int NT = (TI + 1) * TJ;
    switch (stage) {
        case 1: k_ens_stage_f32<TI, TJ, 1><<<grid, NT, 0, s>>>(e); break;
        case 2: k_ens_stage_f32<TI, TJ, 2><<<grid, NT, 0, s>>>(e); break;
        default: k_ens_stage_f32<TI, TJ, 3><<<grid, NT, 0, s>>>(e); break;
    }
    return cudaGetLastError();
}

template <int TI, int TJ>
static int ens_resident_f32() {
    constexpr int NT = (TI + 1) * TJ;
    int n1 = 0, n2 = 0, n3 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_ens_stage_f32<TI, TJ, 1>, NT, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_ens_stage_f32<TI, TJ, 2>, NT, 0) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n3, k_ens_stage_f32<TI, TJ, 3>, NT, 0)) {
        cudaGetLastError();
        return 0;
    }
    return n1 < n2 ? (n1 < n3 ? n1 : n3) : (n2 < n3 ? n2 : n3);
}

int ens_resident_per_sm_f32(int shape) {
    switch (shape) {
        case SHAPE_COLS: {
            int n1 = 0, n2 = 0, n3 = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k_ens_stage_f32_cols<1>, 32 * F32_WARPS, 0) ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_ens_stage_f32_cols<2>, 32 * F32_WARPS, 0) ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n3, k_ens_stage_f32_cols<3>, 32 * F32_WARPS, 0)) {
                cudaGetLastError();
                return 0;
            }
            return std::min(n1, std::min(n2, n3));
        }
        case SHAPE_8x32: return ens_resident_f32<8, 32>();
        case SHAPE_16x32: return ens_resident_f32<16, 32>();
        case SHAPE_8x64: return ens_resident_f32<8, 64>();
        default: return 0;
    }
}

cudaError_t launch_ens_stage_f32(int shape, int stage, const EnsParams &e, int grid,
                                 cudaStream_t s) {
    switch (shape) {
        case SHAPE_COLS:
            switch (stage) {
                case 1: k_ens_stage_f32_cols<1><<<grid, 32 * F32_WARPS, 0, s>>>(e); break;
                case 2: k_ens_stage_f32_cols<2><<<grid, 32 * F32_WARPS, 0, s>>>(e); break;
                default: k_ens_stage_f32_cols<3><<<grid, 32 * F32_WARPS, 0, s>>>(e); break;
            }
            return cudaGetLastError();
        case SHAPE_8x32: return ens_launch_f32<8, 32>(stage, e, grid, s);
        case SHAPE_16x32: return ens_launch_f32<16, 32>(stage, e, grid, s);
        case SHAPE_8x64: return ens_launch_f32<8, 64>(stage, e, grid, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_max_speed_f32(const void *e, const void *hu, const void *hv, const void *B,
                                 int Nx, int Ny, long long pitch, double g,
                                 unsigned long long *slot, int num_sms, cudaStream_t s) {
    k_max_speed_f32<<<grid_for((long long)Nx * Ny, num_sms), 256, 0, s>>>(
        static_cast<const float *>(e), static_cast<const float *>(hu),
        static_cast<const float *>(hv), static_cast<const float *>(B), Nx, Ny, pitch, (float)g,
        slot);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const void *src, const void *add, void *dst, int rows, int cols,
                              long long pitch, int num_sms, cudaStream_t s) {
    k_f64_to_f32<<<grid_for((long long)rows * cols, num_sms), 256, 0, s>>>(
        static_cast<const double *>(src), static_cast<const double *>(add),
        static_cast<float *>(dst), rows, cols, pitch);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const void *src, const void *sub, void *dst, int rows, int cols,
                              long long pitch, int num_sms, cudaStream_t s) {
    k_f32_to_f64<<<grid_for((long long)rows * cols, num_sms), 256, 0, s>>>(
        static_cast<const float *>(src), static_cast<const float *>(sub),
        static_cast<double *>(dst), rows, cols, pitch);
    return cudaGetLastError();
}

cudaError_t launch_fill_ghosts_f32(void *e, void *hu, void *hv, const void *B, int Nx, int Ny,
                                   long long pitch, int bc, cudaStream_t s) {
    const int n = 4 * (Ny + 2 * NG) + 4 * Nx;
    k_fill_ghosts_f32<<<(n + 255) / 256, 256, 0, s>>>(
        static_cast<float *>(e), static_cast<float *>(hu), static_cast<float *>(hv),
        static_cast<const float *>(B), Nx, Ny, pitch, bc);
    return cudaGetLastError();
}

}  // namespace swe
