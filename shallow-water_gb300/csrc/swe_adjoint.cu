// Discrete adjoint with binomial checkpointing (C ABI: swe_adjoint_gauge in
// include/swe_gb300.h), of the FP64 scheme on FP64 contexts and of the FP32-mixed
// scheme on FP32-mixed contexts.
//
// FP32-mixed: the forward (and every recomputation) is the FP32 stage kernel; the VJP
// is the same interface derivative evaluated in FP32 (swe_adjoint_math.cuh is templated
// on the scalar), with the state variable eta = h + B instead of h: the interface reads
// eta directly (so its eta adjoint goes to eta alone, not to B), a positivity clamp
// (eta = B + floor) passes the output adjoint to B, the gauge residual h = eta - B feeds
// both, and the stage-3 weights are the FP32 kernel's n + c (s' - n) with c = fl(2/3).
// At the end dJ/dh0 = dJ/deta0 and dJ/dB (h0 fixed) = the B adjoint + dJ/deta0.  Ghost
// beds must repeat the interior (as the reference's boundary conditions leave them), so
// that a ghost's eta is its source cell's.
//
// Objective: J = sum over steps n = 1..N and gauge cells g of (h^n_g - h_obs^n_g)^2,
// fixed dt.  Gradients: dJ/dh^0, dJ/dhu^0, dJ/dhv^0 and dJ/dB (initial state held fixed).
//
// One adjoint step (transition k -> k+1, U^k in the work buffer):
//  1. recompute the three stages with clamp masks, U^(k+1) into a separate buffer;
//  2. add the gauge source 2 (h - h_obs) of step k+1 to lambda and accumulate J;
//  3. reverse stages 3, 2, 1, each in two passes: k_adj_faces applies the VJP of every
//     x- and y-interface once (swe_adjoint_math.cuh) to the adjoint of the divergence and
//     stores its 14 stencil contributions; k_adj_gather sums, per cell, the contributions
//     of the interfaces whose stencil holds it (ghost slots folded onto the interior
//     cells they mirror, normal momentum negated at reflecting walls).  No atomics: the
//     result does not depend on scheduling.
// States U^k come from a binomial checkpoint schedule over `n_snapshots` stored states,
// chosen by dynamic programming to minimise the number of recomputed forward steps
// (Griewank-Walther binomial checkpointing, cost recursion
// F(n, s) = min_m m + F(n - m, s - 1) + F(m, s)).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "swe_adjoint_math.cuh"
#include "swe_common.cuh"
#include "swe_ctx.h"
#include "swe_launch.h"

namespace swe {
namespace {

constexpr int AFT = 128;  // threads per block of the interface pass
constexpr int AGT = 256;  // threads per block of the gather pass
constexpr int NC = 14;    // contributions per interface: eta(4), qn(4), qt(4), bm, bp

// T = double: FP64 scheme, state (h, hu, hv); T = float: FP32-mixed, state (eta, hu, hv).
template <class T>
struct AdjParams {
    const T *h, *hu, *hv, *B;       // stage source state, bathymetry
    const T *lo_h, *lo_hu, *lo_hv;  // adjoint of the stage output
    const unsigned char *mask;      // positivity clamps of this stage
    T *ls_h, *ls_hu, *ls_hv;        // adjoint of the stage source (written)
    T *ln_h, *ln_hu, *ln_hv;        // adjoint of U^n (stage 3 writes, 2 adds, 1 reads)
    T *gB;                          // dJ/dB (accumulated)
    T *cx, *cy;                     // interface contributions, NC planes each
    long long px, py;               // plane sizes: (Nx + 1) * Ny, Nx * (Ny + 1)
    int Nx, Ny;
    long long pitch;
    int bc;
    T inv_dx, inv_dy, g, dt;
    T kx, ky;  // the stage's source weight x dt x 1/dx (1/dy): divergence to flux adjoint
};

template <class T>
__host__ __device__ constexpr bool eta_state() { return std::is_same<T, float>::value; }

// Weight of the stage source in the stage output, and of U^n in stage 3: the FP64
// kernel's (1.0 / 3.0) U^n + (2.0 / 3.0) (...), the FP32 kernel's n + c (s' - n).
template <class T, int STAGE>
__device__ __forceinline__ T src_weight() {
    if (STAGE == 1) return T(1);
    if (STAGE == 2) return T(0.25);
    return eta_state<T>() ? T(2.f / 3.f) : T(2.0 / 3.0);
}
template <class T>
__device__ __forceinline__ T n_weight3() {
    return eta_state<T>() ? T(1.f - 2.f / 3.f) : T(1.0 / 3.0);
}

// Adjoint of the divergence at interior cell (i, j): cs * dt * lo, zero where the stage
// clamped the depth (its output did not depend on the fluxes there) and outside.
template <class T, int STAGE>
__device__ __forceinline__ void w_at(const AdjParams<T> &a, int i, int j, T w[3]) {
    w[0] = w[1] = w[2] = T(0);
    if (i < 0 || i >= a.Nx || j < 0 || j >= a.Ny) return;
    const long long k = (long long)(i + NG) * a.pitch + (j + NG);
    if (a.mask[k]) return;
    const T f = src_weight<T, STAGE>() * a.dt;
    w[0] = f * a.lo_h[k];
    w[1] = f * a.lo_hu[k];
    w[2] = f * a.lo_hv[k];
}

// The stage output's adjoint at interior cell (i, j), zero where the stage clamped the
// depth and outside; k_adj_faces scales its differences by the stage's kx or ky.
template <class T>
__device__ __forceinline__ void lo_at(const AdjParams<T> &a, int i, int j, T l[3]) {
    l[0] = l[1] = l[2] = T(0);
    if (i < 0 || i >= a.Nx || j < 0 || j >= a.Ny) return;
    const long long k = (long long)(i + NG) * a.pitch + (j + NG);
    if (a.mask[k]) return;
    l[0] = a.lo_h[k];
    l[1] = a.lo_hu[k];
    l[2] = a.lo_hv[k];
}

// One interface per thread.  DIR 0: x-interface f in [-1, Nx - 1] between rows f and
// f + 1 at column j; DIR 1: y-interface f in [-1, Ny - 1] between columns f and f + 1 at
// row i.  The stencil is staged exactly as the forward kernel stages it: the state of
// ghost cells from the mirrored (reflecting, normal momentum negated) or clamped
// (transmissive) interior cell, B where it lies, ghosts included.
// Five 128-thread CTAs per SM (at most 102 registers; the VJP needs 104 uncapped and does
// not spill at 102): 1% faster than four; six and seven CTAs spill and are slower.
#ifndef SWE_ADJ_FACES_MIN_BLOCKS
#define SWE_ADJ_FACES_MIN_BLOCKS 5
#endif
template <class T, int STAGE, int DIR>
__global__ void __launch_bounds__(AFT, SWE_ADJ_FACES_MIN_BLOCKS) k_adj_faces(const AdjParams<T> a) {
    const int t = blockIdx.x * AFT + threadIdx.x;
    const int along = DIR == 0 ? a.Ny : a.Ny + 1;  // contiguous index range
    if (t >= along) return;
    const int f = DIR == 0 ? (int)blockIdx.y - 1 : t - 1;  // interface index
    const int o = DIR == 0 ? t : (int)blockIdx.y;          // the other coordinate
    const long long P = a.pitch;
    adj::FaceIn<T> in;
    for (int q = 0; q < 4; ++q) {
        const int c = f - 1 + q;  // stencil cell along the normal
        bool fl;
        const int m = map_coord(c, DIR == 0 ? a.Nx : a.Ny, a.bc, fl);
        const long long ks = DIR == 0 ? (long long)(m + NG) * P + (o + NG)
                                      : (long long)(o + NG) * P + (m + NG);
        const int cb = clamp_int(c + NG, 0, (DIR == 0 ? a.Nx : a.Ny) + 3);
        const long long kb = DIR == 0 ? (long long)cb * P + (o + NG) : (long long)(o + NG) * P + cb;
        const T b = a.B[kb];
        const T qn = DIR == 0 ? a.hu[ks] : a.hv[ks];
        if (eta_state<T>()) {  // the FP32 kernel's ghost: its source's depth over its own bed
            const T bs = a.B[ks], e = a.h[ks];
            in.e[q] = (b == bs) ? e : (e - bs) + b;
        } else {
            in.e[q] = a.h[ks] + b;
        }
        in.n[q] = fl ? -qn : qn;
        in.t[q] = DIR == 0 ? a.hv[ks] : a.hu[ks];
        if (q == 1) in.bm = b;
        if (q == 2) in.bp = b;
    }
    T lm[3], lp[3];
    if (DIR == 0) {
        lo_at(a, f, o, lm);
        lo_at(a, f + 1, o, lp);
    } else {
        lo_at(a, o, f, lm);
        lo_at(a, o, f + 1, lp);
    }
    const T k = DIR == 0 ? a.kx : a.ky;
    const int n = DIR == 0 ? 1 : 2, tg = DIR == 0 ? 2 : 1;  // normal / tangential field
    adj::FaceOut<T> d;
    d.fh = k * (lp[0] - lm[0]);
    d.fqt = k * (lp[tg] - lm[tg]);
    d.fqn_m = -k * lm[n];
    d.fqn_p = k * lp[n];
    adj::FaceIn<T> ad;
    adj::face_vjp(in, a.g, T(EPS), d, ad);
    T *C = DIR == 0 ? a.cx : a.cy;
    const long long pl = DIR == 0 ? a.px : a.py;
    const long long idx = DIR == 0 ? (long long)(f + 1) * a.Ny + o : (long long)o * (a.Ny + 1) + (f + 1);
    for (int q = 0; q < 4; ++q) {
        C[(q)*pl + idx] = ad.e[q];
        C[(4 + q) * pl + idx] = ad.n[q];
        C[(8 + q) * pl + idx] = ad.t[q];
    }
    C[12 * pl + idx] = ad.bm;
    C[13 * pl + idx] = ad.bp;
}

// Interior coordinate a plus the ghost coordinates whose values are copies of cell a
// (reflecting: mirrored, normal component negated; transmissive: clamped).
__device__ __forceinline__ int virtual_coords(int a, int N, int bc, int *v, bool *fl) {
    int n = 0;
    v[n] = a;
    fl[n++] = false;
    if (bc == BC_REFLECTING) {
        if (a <= 1) {
            v[n] = -1 - a;
            fl[n++] = true;
        }
        if (a >= N - 2) {
            v[n] = 2 * N - 1 - a;
            fl[n++] = true;
        }
    } else {
        if (a == 0) {
            v[n] = -1;
            fl[n++] = false;
            v[n] = -2;
            fl[n++] = false;
        }
        if (a == N - 1) {
            v[n] = N;
            fl[n++] = false;
            v[n] = N + 1;
            fl[n++] = false;
        }
    }
    return n;
}

// Sums, for interior cell a along one direction (rows for DIR 0, columns for DIR 1), the
// contributions of the interfaces whose stencil holds a or a ghost copy of it.
template <class T, int DIR>
__device__ __forceinline__ void gather_dir(const AdjParams<T> &a, int ca, int other, T &acc_h,
                                           T &acc_qn, T &acc_qt, T &acc_B) {
    const int N = DIR == 0 ? a.Nx : a.Ny;
    const T *C = DIR == 0 ? a.cx : a.cy;
    const long long pl = DIR == 0 ? a.px : a.py;
    auto at = [&](int f) {  // linear index of interface f (valid range [-1, N - 1])
        return DIR == 0 ? (long long)(f + 1) * a.Ny + other : (long long)other * (a.Ny + 1) + (f + 1);
    };
    int v[5];
    bool fl[5];
    const int nv = virtual_coords(ca, N, a.bc, v, fl);
    for (int q = 0; q < nv; ++q) {
        for (int k = 0; k < 4; ++k) {
            const int f = v[q] + 1 - k;  // interface whose stencil slot k is cell v
            if (f < -1 || f > N - 1) continue;
            const long long x = at(f);
            const T ce = C[k * pl + x], cn = C[(4 + k) * pl + x];
            acc_h += ce;
            acc_qn += fl[q] ? -cn : cn;
            acc_qt += C[(8 + k) * pl + x];
        }
        const int fm = v[q], fp = v[q] - 1;  // interfaces with cell v as minus / plus side
        if (fm >= -1 && fm <= N - 1) acc_B += C[12 * pl + at(fm)];
        if (fp >= -1 && fp <= N - 1) acc_B += C[13 * pl + at(fp)];
    }
}

// Per interior cell: adjoint of the stage source and of U^n, and dJ/dB.
template <class T, int STAGE>
__global__ void __launch_bounds__(AGT) k_adj_gather(const AdjParams<T> a) {
    const int cj = blockIdx.x * AGT + threadIdx.x, ci = blockIdx.y;
    if (cj >= a.Ny) return;
    const T cs = src_weight<T, STAGE>();
    T acc_h = T(0), acc_hu = T(0), acc_hv = T(0), acc_B = T(0);
    gather_dir<T, 0>(a, ci, cj, acc_h, acc_hu, acc_hv, acc_B);
    gather_dir<T, 1>(a, cj, ci, acc_h, acc_hv, acc_hu, acc_B);
    if (!eta_state<T>()) acc_B += acc_h;  // every interface read eta = h + B
    const long long k = (long long)(ci + NG) * a.pitch + (cj + NG);
    const bool m = a.mask[k];
    // a clamped FP32 cell is eta = B + floor: its eta adjoint goes to B
    if (eta_state<T>() && m) acc_B += a.lo_h[k];
    const T l0 = m ? T(0) : a.lo_h[k], l1 = m ? T(0) : a.lo_hu[k], l2 = m ? T(0) : a.lo_hv[k];
    T o0 = acc_h + cs * l0, o1 = acc_hu + cs * l1, o2 = acc_hv + cs * l2;
    if (STAGE == 3) {  // the forward's weight of U^n
        const T wn = n_weight3<T>();
        a.ln_h[k] = wn * l0;
        a.ln_hu[k] = wn * l1;
        a.ln_hv[k] = wn * l2;
    } else if (STAGE == 2) {
        a.ln_h[k] += T(0.75) * l0;
        a.ln_hu[k] += T(0.75) * l1;
        a.ln_hv[k] += T(0.75) * l2;
    } else {
        o0 += a.ln_h[k];
        o1 += a.ln_hu[k];
        o2 += a.ln_hv[k];
    }
    a.ls_h[k] = o0;
    a.ls_hu[k] = o1;
    a.ls_hv[k] = o2;
    a.gB[k] += acc_B;
}

// Single-pass reverse of one stage for a TI x TJ tile (the FP32 path): the tile's
// stage source (halo 3) and divergence adjoint (halo 2) are staged in shared memory,
// every x- and y-interface whose stencil holds a tile cell is reversed there (TI + 3
// rows of x-interfaces, TJ + 3 columns of y-interfaces: 1.23 interface VJPs per cell,
// against 1.0 in the two-pass form), and each cell gathers its contributions from
// shared memory in the two-pass gather's order, so the results are bitwise the same.
// The interface contributions never reach HBM: about 70 bytes per cell and stage move
// instead of about 300, which is what bounds the FP32 reverse sweep.
#ifndef SWE_ADJ_TILE_I
#define SWE_ADJ_TILE_I 8
#endif
constexpr int ATI = SWE_ADJ_TILE_I, ATJ = 32, ATT = ATI * ATJ;
constexpr int AT_MIN_BLOCKS = 1024 / ATT;  // 64 registers a thread

template <class T>
struct AdjTile {
    T st[4][ATI + 6][ATJ + 6];         // eta (or h + B), qn-x (hu), qn-y (hv), B; halo 3
    T w[3][ATI + 4][ATJ + 4];          // cs dt lo, zero outside and where clamped; halo 2
    T cx[NC][ATI + 3][ATJ];            // x-interfaces i0-2 .. i0+TI
    T cy[NC][ATI][ATJ + 3];            // y-interfaces j0-2 .. j0+TJ
};

template <class T, int STAGE>
__global__ void __launch_bounds__(ATT, AT_MIN_BLOCKS) k_adj_tile(const AdjParams<T> a) {
    extern __shared__ __align__(16) unsigned char adj_smem[];
    AdjTile<T> &t = *reinterpret_cast<AdjTile<T> *>(adj_smem);
    const int tid = threadIdx.x;
    const int i0 = blockIdx.y * ATI, j0 = blockIdx.x * ATJ;
    const long long P = a.pitch;
    // stage source, as k_adj_faces reads each stencil cell
    for (int e = tid; e < (ATI + 6) * (ATJ + 6); e += ATT) {
        const int r = e / (ATJ + 6), c = e - r * (ATJ + 6);
        const int i = i0 - 3 + r, j = j0 - 3 + c;
        T ev = T(0), u = T(0), v = T(0), b = T(0);
        if (i >= -2 && i <= a.Nx + 1 && j >= -2 && j <= a.Ny + 1) {
            bool fx, fy;
            const int mi = map_coord(i, a.Nx, a.bc, fx), mj = map_coord(j, a.Ny, a.bc, fy);
            const long long ks = (long long)(mi + NG) * P + (mj + NG);
            const long long kb = (long long)clamp_int(i + NG, 0, a.Nx + 3) * P +
                                 clamp_int(j + NG, 0, a.Ny + 3);
            b = a.B[kb];
            if (eta_state<T>()) {
                const T bs = a.B[ks], e0 = a.h[ks];
                ev = (b == bs) ? e0 : (e0 - bs) + b;
            } else {
                ev = a.h[ks] + b;
            }
            u = fx ? -a.hu[ks] : a.hu[ks];
            v = fy ? -a.hv[ks] : a.hv[ks];
        }
        t.st[0][r][c] = ev;
        t.st[1][r][c] = u;
        t.st[2][r][c] = v;
        t.st[3][r][c] = b;
    }
    for (int e = tid; e < (ATI + 4) * (ATJ + 4); e += ATT) {
        const int r = e / (ATJ + 4), c = e - r * (ATJ + 4);
        T w[3];
        w_at<T, STAGE>(a, i0 - 2 + r, j0 - 2 + c, w);
        t.w[0][r][c] = w[0];
        t.w[1][r][c] = w[1];
        t.w[2][r][c] = w[2];
    }
    __syncthreads();
    const T g = a.g, eps = T(EPS);
    // x-interfaces f = i0 - 2 + ar between rows f and f + 1, column j0 + c
    for (int e = tid; e < (ATI + 3) * ATJ; e += ATT) {
        const int ar = e / ATJ, c = e - ar * ATJ;
        const int f = i0 - 2 + ar;
        if (f < -1 || f > a.Nx - 1 || j0 + c >= a.Ny) continue;
        adj::FaceIn<T> in;
        for (int q = 0; q < 4; ++q) {  // box row of stencil cell f - 1 + q: ar + q
            in.e[q] = t.st[0][ar + q][c + 3];
            in.n[q] = t.st[1][ar + q][c + 3];
            in.t[q] = t.st[2][ar + q][c + 3];
        }
        in.bm = t.st[3][ar + 1][c + 3];
        in.bp = t.st[3][ar + 2][c + 3];
        adj::FaceOut<T> d;  // w rows of cells f, f + 1: ar, ar + 1
        d.fh = a.inv_dx * (t.w[0][ar + 1][c + 2] - t.w[0][ar][c + 2]);
        d.fqt = a.inv_dx * (t.w[2][ar + 1][c + 2] - t.w[2][ar][c + 2]);
        d.fqn_m = -a.inv_dx * t.w[1][ar][c + 2];
        d.fqn_p = a.inv_dx * t.w[1][ar + 1][c + 2];
        adj::FaceIn<T> ad;
        adj::face_vjp(in, g, eps, d, ad);
        for (int q = 0; q < 4; ++q) {
            t.cx[q][ar][c] = ad.e[q];
            t.cx[4 + q][ar][c] = ad.n[q];
            t.cx[8 + q][ar][c] = ad.t[q];
        }
        t.cx[12][ar][c] = ad.bm;
        t.cx[13][ar][c] = ad.bp;
    }
    // y-interfaces f = j0 - 2 + bc between columns f and f + 1, row i0 + r
    for (int e = tid; e < ATI * (ATJ + 3); e += ATT) {
        const int r = e / (ATJ + 3), bc = e - r * (ATJ + 3);
        const int f = j0 - 2 + bc;
        if (f < -1 || f > a.Ny - 1 || i0 + r >= a.Nx) continue;
        adj::FaceIn<T> in;
        for (int q = 0; q < 4; ++q) {
            in.e[q] = t.st[0][r + 3][bc + q];
            in.n[q] = t.st[2][r + 3][bc + q];
            in.t[q] = t.st[1][r + 3][bc + q];
        }
        in.bm = t.st[3][r + 3][bc + 1];
        in.bp = t.st[3][r + 3][bc + 2];
        adj::FaceOut<T> d;
        d.fh = a.inv_dy * (t.w[0][r + 2][bc + 1] - t.w[0][r + 2][bc]);
        d.fqt = a.inv_dy * (t.w[1][r + 2][bc + 1] - t.w[1][r + 2][bc]);
        d.fqn_m = -a.inv_dy * t.w[2][r + 2][bc];
        d.fqn_p = a.inv_dy * t.w[2][r + 2][bc + 1];
        adj::FaceIn<T> ad;
        adj::face_vjp(in, g, eps, d, ad);
        for (int q = 0; q < 4; ++q) {
            t.cy[q][r][bc] = ad.e[q];
            t.cy[4 + q][r][bc] = ad.n[q];
            t.cy[8 + q][r][bc] = ad.t[q];
        }
        t.cy[12][r][bc] = ad.bm;
        t.cy[13][r][bc] = ad.bp;
    }
    __syncthreads();
    const int r = tid / ATJ, c = tid - r * ATJ;
    const int ci = i0 + r, cj = j0 + c;
    if (ci >= a.Nx || cj >= a.Ny) return;
    T acc_h = T(0), acc_hu = T(0), acc_hv = T(0), acc_B = T(0);
    // gather_dir<T, 0> and <T, 1> with the contributions read from shared memory
    for (int dir = 0; dir < 2; ++dir) {
        const int ca = dir == 0 ? ci : cj, N = dir == 0 ? a.Nx : a.Ny;
        const int base = dir == 0 ? i0 - 2 : j0 - 2;
        T &acc_n = dir == 0 ? acc_hu : acc_hv, &acc_t = dir == 0 ? acc_hv : acc_hu;
        int v[5];
        bool fl[5];
        const int nv = virtual_coords(ca, N, a.bc, v, fl);
        auto C = [&](int q, int f) -> T {
            return dir == 0 ? t.cx[q][f - base][c] : t.cy[q][r][f - base];
        };
        for (int q = 0; q < nv; ++q) {
            for (int k = 0; k < 4; ++k) {
                const int f = v[q] + 1 - k;
                if (f < -1 || f > N - 1) continue;
                const T ce = C(k, f), cn = C(4 + k, f);
                acc_h += ce;
                if (!eta_state<T>()) acc_B += ce;
                acc_n += fl[q] ? -cn : cn;
                acc_t += C(8 + k, f);
            }
            const int fm = v[q], fp = v[q] - 1;
            if (fm >= -1 && fm <= N - 1) acc_B += C(12, fm);
            if (fp >= -1 && fp <= N - 1) acc_B += C(13, fp);
        }
    }
    const T cs = src_weight<T, STAGE>();
    const long long k = (long long)(ci + NG) * P + (cj + NG);
    const bool m = a.mask[k];
    if (eta_state<T>() && m) acc_B += a.lo_h[k];
    const T l0 = m ? T(0) : a.lo_h[k], l1 = m ? T(0) : a.lo_hu[k], l2 = m ? T(0) : a.lo_hv[k];
    T o0 = acc_h + cs * l0, o1 = acc_hu + cs * l1, o2 = acc_hv + cs * l2;
    if (STAGE == 3) {
        const T wn = n_weight3<T>();
        a.ln_h[k] = wn * l0;
        a.ln_hu[k] = wn * l1;
        a.ln_hv[k] = wn * l2;
    } else if (STAGE == 2) {
        a.ln_h[k] += T(0.75) * l0;
        a.ln_hu[k] += T(0.75) * l1;
        a.ln_hv[k] += T(0.75) * l2;
    } else {
        o0 += a.ln_h[k];
        o1 += a.ln_hu[k];
        o2 += a.ln_hv[k];
    }
    a.ls_h[k] = o0;
    a.ls_hu[k] = o1;
    a.ls_hv[k] = o2;
    a.gB[k] += acc_B;
}

// Gauge source of one step: lambda_h[g] += 2 (h_g - obs_g), J += sum (h_g - obs_g)^2,
// one thread in gauge order (deterministic, duplicates allowed).
// FP32-mixed: h = eta - B in FP64, lambda_eta += 2 (h - obs) and lambda_B -= 2 (h - obs).
template <class T>
__global__ void k_gauge(const T *h, const T *B, long long P, const int *gi, const int *gj,
                        int ng, const double *obs, T *lam_h, T *gB, double *J) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int q = 0; q < ng; ++q) {
        const long long k = (long long)(gi[q] + NG) * P + (gj[q] + NG);
        const double hk = eta_state<T>() ? (double)h[k] - (double)B[k] : (double)h[k];
        const double r = hk - obs[q];
        s += r * r;
        if (!lam_h) continue;  // objective only
        lam_h[k] += (T)(2.0 * r);
        if (eta_state<T>()) gB[k] -= (T)(2.0 * r);
    }
    *J += s;
}

// dJ/dB with h0 held fixed, widened: B adjoint + the eta0 adjoint (FP32-mixed).
__global__ void k_grad_b_f32(const float *gB, const float *lam_e, double *out, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x)
        out[t] = (double)gB[t] + (double)lam_e[t];
}

__global__ void k_widen(const float *src, double *out, size_t n) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x)
        out[t] = (double)src[t];
}

template <class T>
struct Adj {
    swe_ctx *c;
    size_t fe;  // elements per field
    T *snap;
    int S;
    T *W[3], *Un1[3], *lam[3], *lamA[3], *lamB[3], *ln[3], *gB;
    T *cx, *cy;  // interface contributions of the stage being reversed
    bool tape = false;            // every state and every step's stage states kept
    int seg_len = 0;              // segmented schedule: steps per segment (0: not used)
    int nseg = 0;                 // segmented schedule: number of segments
    T *tU1 = nullptr, *tU2 = nullptr;  // tape: U^(1), U^(2) of step k at 3 k fields
    unsigned char *tmask = nullptr;    // tape: clamp masks of step k at 3 k fields
    unsigned char *mask[3];
    int *gi, *gj;
    double *obs, *J;
    unsigned long long *speed;
    int ng;
    double dt;
    std::vector<std::vector<int>> split;  // optimal first advance, [n][s]
    long long fwd_steps = 0;
};

#define ACK(call)                                  \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return e_;          \
    } while (0)

template <class T>
StageParams fwd_params(const Adj<T> &A) {
    const swe_ctx *c = A.c;
    StageParams sp{};
    sp.B = c->B;
    sp.Nx = c->p.Nx;
    sp.Ny = c->p.Ny;
    sp.pitch = c->pitch;
    sp.bc = c->p.bc;
    sp.inv_dx = c->inv_dx;
    sp.inv_dy = c->inv_dy;
    sp.kx = pow2_exponent(c->inv_dx);
    sp.ky = pow2_exponent(c->inv_dy);
    sp.g = c->p.g;
    sp.half_g = 0.5 * c->p.g;
    sp.gf = (float)sp.g;
    sp.half_gf = (float)sp.half_g;
    sp.inv_dxf = (float)sp.inv_dx;
    sp.inv_dyf = (float)sp.inv_dy;
    sp.cfl_min_dxdy = c->cfl_min_dxdy;
    sp.dt_fixed = A.dt;
    sp.speed = A.speed;  // scratch slots: the context's adaptive-dt slots stay untouched
    sp.slot_read = 0;
    sp.slot_write = 1;
    sp.flags = c->flags;
    return sp;
}

template <class T>
cudaError_t launch_fwd_stage(int stage, const StageParams &sp, cudaStream_t s) {
    if (eta_state<T>()) return launch_stage_f32(stage, sp, nullptr, s);
    return launch_stage_f64(stage, sp, nullptr, s);
}

// One forward step W -> out (out may be W) with the stage states in U1, U2 and the
// clamp masks in mk[0..2] (null: not kept).
template <class T>
cudaError_t forward_step_into(Adj<T> &A, T *const *W, T *const *out, T *const *U1,
                              T *const *U2, unsigned char *const *mk) {
    swe_ctx *c = A.c;
    StageParams sp = fwd_params(A);
    sp.hn = W[0]; sp.hun = W[1]; sp.hvn = W[2];
    sp.hs = W[0]; sp.hus = W[1]; sp.hvs = W[2];
    sp.ho = U1[0]; sp.huo = U1[1]; sp.hvo = U1[2];
    sp.mask = mk[0];
    ACK(launch_fwd_stage<T>(1, sp, c->stream));
    sp.hs = U1[0]; sp.hus = U1[1]; sp.hvs = U1[2];
    sp.ho = U2[0]; sp.huo = U2[1]; sp.hvo = U2[2];
    sp.mask = mk[1];
    ACK(launch_fwd_stage<T>(2, sp, c->stream));
    sp.hs = U2[0]; sp.hus = U2[1]; sp.hvs = U2[2];
    sp.ho = out[0]; sp.huo = out[1]; sp.hvo = out[2];
    sp.mask = mk[2];
    ACK(launch_fwd_stage<T>(3, sp, c->stream));
    c->launches += 3;
    ++A.fwd_steps;
    return cudaSuccess;
}

template <class T>
void ctx_stage_buffers(const swe_ctx *c, T **U1, T **U2) {
    for (int f = 0; f < 3; ++f) {
        U1[f] = static_cast<T *>(c->U1[f]);
        U2[f] = static_cast<T *>(c->U2[f]);
    }
}

// One forward step W -> out through the context's stage buffers; masks optional.
template <class T>
cudaError_t forward_step(Adj<T> &A, T *const *W, T *const *out, bool masks) {
    T *U1[3], *U2[3];
    ctx_stage_buffers(A.c, U1, U2);
    unsigned char *none[3] = {nullptr, nullptr, nullptr};
    return forward_step_into(A, W, out, U1, U2, masks ? A.mask : none);
}

template <class T>
cudaError_t launch_adj(Adj<T> &A, int stage, T *const *state, T *const *lo,
                       const unsigned char *mask, T *const *ls) {
    swe_ctx *c = A.c;
    AdjParams<T> p{};
    p.h = state[0]; p.hu = state[1]; p.hv = state[2];
    p.B = static_cast<const T *>(c->B);
    p.lo_h = lo[0]; p.lo_hu = lo[1]; p.lo_hv = lo[2];
    p.mask = mask;
    p.ls_h = ls[0]; p.ls_hu = ls[1]; p.ls_hv = ls[2];
    p.ln_h = A.ln[0]; p.ln_hu = A.ln[1]; p.ln_hv = A.ln[2];
    p.gB = A.gB;
    p.Nx = c->p.Nx;
    p.Ny = c->p.Ny;
    p.pitch = c->pitch;
    p.bc = c->p.bc;
    p.inv_dx = (T)c->inv_dx;
    p.inv_dy = (T)c->inv_dy;
    p.g = (T)c->p.g;
    p.dt = (T)A.dt;
    {
        const double w = stage == 1 ? 1.0 : (stage == 2 ? 0.25 : 2.0 / 3.0);
        p.kx = (T)(w * A.dt * c->inv_dx);
        p.ky = (T)(w * A.dt * c->inv_dy);
    }
    p.cx = A.cx;
    p.cy = A.cy;
    p.px = (long long)(c->p.Nx + 1) * c->p.Ny;
    p.py = (long long)c->p.Nx * (c->p.Ny + 1);
    if constexpr (eta_state<T>()) {  // FP32: the single-pass tile kernel (memory-bound otherwise)
        const int smem = (int)sizeof(AdjTile<T>);
        static bool opted[4];
        if (!opted[stage]) {
            auto kern = stage == 1 ? k_adj_tile<T, 1> : (stage == 2 ? k_adj_tile<T, 2> : k_adj_tile<T, 3>);
            ACK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            opted[stage] = true;
        }
        const dim3 gt((c->p.Ny + ATJ - 1) / ATJ, (c->p.Nx + ATI - 1) / ATI);
        if (stage == 1)
            k_adj_tile<T, 1><<<gt, ATT, smem, c->stream>>>(p);
        else if (stage == 2)
            k_adj_tile<T, 2><<<gt, ATT, smem, c->stream>>>(p);
        else
            k_adj_tile<T, 3><<<gt, ATT, smem, c->stream>>>(p);
        ++c->launches;
        return cudaGetLastError();
    }
    const dim3 gx((c->p.Ny + AFT - 1) / AFT, c->p.Nx + 1), gy((c->p.Ny + 1 + AFT - 1) / AFT, c->p.Nx);
    const dim3 gg((c->p.Ny + AGT - 1) / AGT, c->p.Nx);
    switch (stage) {
        case 1:
            k_adj_faces<T, 1, 0><<<gx, AFT, 0, c->stream>>>(p);
            k_adj_faces<T, 1, 1><<<gy, AFT, 0, c->stream>>>(p);
            k_adj_gather<T, 1><<<gg, AGT, 0, c->stream>>>(p);
            break;
        case 2:
            k_adj_faces<T, 2, 0><<<gx, AFT, 0, c->stream>>>(p);
            k_adj_faces<T, 2, 1><<<gy, AFT, 0, c->stream>>>(p);
            k_adj_gather<T, 2><<<gg, AGT, 0, c->stream>>>(p);
            break;
        default:
            k_adj_faces<T, 3, 0><<<gx, AFT, 0, c->stream>>>(p);
            k_adj_faces<T, 3, 1><<<gy, AFT, 0, c->stream>>>(p);
            k_adj_gather<T, 3><<<gg, AGT, 0, c->stream>>>(p);
            break;
    }
    c->launches += 2;
    ++c->launches;
    return cudaGetLastError();
}

template <class T>
cudaError_t gauge_source(Adj<T> &A, const T *h, int k) {
    swe_ctx *c = A.c;
    k_gauge<T><<<1, 32, 0, c->stream>>>(h, static_cast<const T *>(c->B), c->pitch, A.gi, A.gj,
                                        A.ng, A.obs + (size_t)k * A.ng, A.lam[0], A.gB, A.J);
    ++c->launches;
    return cudaGetLastError();
}

// Adjoint of step k (W holds U^k; lam holds the adjoint of U^(k+1) before its source).
template <class T>
cudaError_t adjoint_step(Adj<T> &A, int k) {
    ACK(forward_step(A, A.W, A.Un1, true));
    T *U1[3], *U2[3];
    ctx_stage_buffers(A.c, U1, U2);
    ACK(gauge_source(A, A.Un1[0], k));
    ACK(launch_adj(A, 3, U2, A.lam, A.mask[2], A.lamA));
    ACK(launch_adj(A, 2, U1, A.lamA, A.mask[1], A.lamB));
    ACK(launch_adj(A, 1, A.W, A.lamB, A.mask[0], A.lam));
    return cudaSuccess;
}

template <class T>
cudaError_t copy_state(Adj<T> &A, T *const *dst, T *const *src) {
    for (int f = 0; f < 3; ++f)
        ACK(cudaMemcpyAsync(dst[f], src[f], A.fe * sizeof(T), cudaMemcpyDeviceToDevice,
                            A.c->stream));
    return cudaSuccess;
}

template <class T>
T *slot_field(Adj<T> &A, int slot, int f) { return A.snap + ((size_t)slot * 3 + f) * A.fe; }

template <class T>
cudaError_t load_slot(Adj<T> &A, int slot) {
    T *src[3] = {slot_field(A, slot, 0), slot_field(A, slot, 1), slot_field(A, slot, 2)};
    return copy_state(A, A.W, src);
}

template <class T>
cudaError_t store_slot(Adj<T> &A, int slot) {
    T *dst[3] = {slot_field(A, slot, 0), slot_field(A, slot, 1), slot_field(A, slot, 2)};
    return copy_state(A, dst, A.W);
}

template <class T>
T *tape_field(T *base, Adj<T> &A, int k, int f) { return base + ((size_t)k * 3 + f) * A.fe; }

// Steps [l, l + m) from U^l in snapshot slot `base`: one forward sweep keeps U^(l+j) in
// slot base + j and the stage states and clamp masks of step l + j at tape position j;
// the reverse sweep over them then recomputes nothing.  Tape mode is this over all steps
// (l = 0, base = 0); the segmented schedule runs it once per segment.
template <class T>
cudaError_t tape_and_reverse(Adj<T> &A, int l, int m, int base) {
    for (int j = 0; j < m; ++j) {
        T *W[3], *out[3], *U1[3], *U2[3];
        unsigned char *mk[3];
        for (int f = 0; f < 3; ++f) {
            W[f] = slot_field(A, base + j, f);
            out[f] = slot_field(A, base + j + 1, f);
            U1[f] = tape_field(A.tU1, A, j, f);
            U2[f] = tape_field(A.tU2, A, j, f);
            mk[f] = A.tmask + ((size_t)j * 3 + f) * A.fe;
        }
        ACK(forward_step_into(A, W, out, U1, U2, mk));
    }
    for (int j = m - 1; j >= 0; --j) {
        T *Wk[3], *U1[3], *U2[3];
        const unsigned char *mk[3];
        for (int f = 0; f < 3; ++f) {
            Wk[f] = slot_field(A, base + j, f);
            U1[f] = tape_field(A.tU1, A, j, f);
            U2[f] = tape_field(A.tU2, A, j, f);
            mk[f] = A.tmask + ((size_t)j * 3 + f) * A.fe;
        }
        ACK(gauge_source(A, slot_field(A, base + j + 1, 0), l + j));
        ACK(launch_adj(A, 3, U2, A.lam, mk[2], A.lamA));
        ACK(launch_adj(A, 2, U1, A.lamA, mk[1], A.lamB));
        ACK(launch_adj(A, 1, Wk, A.lamB, mk[0], A.lam));
    }
    return cudaSuccess;
}

template <class T>
cudaError_t taped(Adj<T> &A, int n) { return tape_and_reverse(A, 0, n, 0); }

// Segmented schedule: the steps are cut into nseg segments of L steps, counted from the
// end (the first segment takes the remainder), so that the last segment is a whole one.
// A first sweep stores the start of segment s in snapshot slot s, up to the last
// segment's start; each segment, last first, is then recomputed once from its snapshot
// with its stage states taped (slots A.nseg + 1 + j), and reversed.  Every step is
// advanced twice (the sweep and its segment's taped recomputation), except the last
// segment's L, which are advanced once; memory holds ceil(n / L) + 1 snapshots and a tape
// of L steps.
template <class T>
cudaError_t segmented(Adj<T> &A, int n) {
    const int L = A.seg_len;
    const int last = A.nseg - 1;
    auto start = [&](int sg) { return sg == 0 ? 0 : n - (A.nseg - sg) * L; };
    int next = 1;
    for (int k = 0; k < start(last); ++k) {
        ACK(forward_step(A, A.W, A.W, false));
        if (k + 1 == start(next)) ACK(store_slot(A, next++));
    }
    const int base = A.nseg + 1;
    for (int sg = last; sg >= 0; --sg) {
        const int l = start(sg), m = start(sg + 1) - l;
        T *src[3] = {slot_field(A, sg, 0), slot_field(A, sg, 1), slot_field(A, sg, 2)};
        T *dst[3] = {slot_field(A, base, 0), slot_field(A, base, 1), slot_field(A, base, 2)};
        ACK(copy_state(A, dst, src));
        ACK(tape_and_reverse(A, l, m, base));
    }
    return cudaSuccess;
}

// Adjoint of steps [l, l+n) with U^l in `slot` and s free snapshot slots.
template <class T>
cudaError_t reverse(Adj<T> &A, int l, int n, int slot, int s) {
    while (true) {
        if (n == 1) {
            ACK(load_slot(A, slot));
            return adjoint_step(A, l);
        }
        if (s == 0) {
            ACK(load_slot(A, slot));
            for (int q = 0; q < n - 1; ++q) ACK(forward_step(A, A.W, A.W, false));
            ACK(adjoint_step(A, l + n - 1));
            --n;
            continue;
        }
        const int m = A.split[n][s];
        ACK(load_slot(A, slot));
        for (int q = 0; q < m; ++q) ACK(forward_step(A, A.W, A.W, false));
        const int fresh = A.S - s + 1;
        ACK(store_slot(A, fresh));
        ACK(reverse(A, l + m, n - m, fresh, s - 1));
        n = m;
    }
}

// split[n][s] minimising F(n, s) = m + F(n - m, s - 1) + F(m, s); F(1, s) = 0,
// F(n, 0) = n (n - 1) / 2.  With s >= n - 1, storing every state (m = 1) is optimal.
template <class T>
void build_schedule(Adj<T> &A, int N, int S) {
    A.split.assign(N + 1, std::vector<int>(S + 1, 1));
    std::vector<std::vector<long long>> F(N + 1, std::vector<long long>(S + 1, 0));
    for (int n = 2; n <= N; ++n) {
        F[n][0] = F[n - 1][0] + (n - 1);
        A.split[n][0] = n - 1;
    }
    for (int s = 1; s <= S; ++s) {
        for (int n = 2; n <= N; ++n) {
            if (s >= n - 1) {
                F[n][s] = n - 1;
                A.split[n][s] = 1;
                continue;
            }
            long long best = -1;
            int bm = 1;
            for (int m = 1; m < n; ++m) {
                const long long cost = m + F[n - m][s - 1] + F[m][s];
                if (best < 0 || cost < best) {
                    best = cost;
                    bm = m;
                }
            }
            F[n][s] = best;
            A.split[n][s] = bm;
        }
    }
}

// Sum of the per-step gauge sums in reverse step order, the order in which the adjoint's
// reverse sweep accumulates J.
__global__ void k_sum_reverse(const double *Jk, int n, double *J) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int k = n - 1; k >= 0; --k) s += Jk[k];
    *J = s;
}

// The objective alone (no gradient): one forward sweep from the context's state through
// the context's stage buffers, each step's gauge sum kept, then summed in the adjoint's
// order.  The same stage kernels, gauge sums and order as a gradient call, so J is
// bitwise that call's J; central finite differences of it check the gradient.
template <class T>
int run_objective(swe_ctx *c, int n_steps, double dt, int n_gauges, const int *gauge_i,
                  const int *gauge_j, const double *h_obs, double *J, double *ms) {
    Adj<T> A;
    A.c = c;
    A.fe = c->field_elems;
    A.ng = n_gauges;
    A.dt = dt;
    const size_t fb = (A.fe * sizeof(T) + 255) / 256 * 256;
    const size_t nobs = (size_t)n_steps * n_gauges + 1;
    const size_t bytes = 3 * fb + 2 * 256 * (((size_t)n_gauges + 1) * sizeof(int) / 256 + 1) +
                         (nobs * sizeof(double) + 255) / 256 * 256 + 512 +
                         ((size_t)n_steps * sizeof(double) + 255) / 256 * 256;
    char *base = nullptr;
    if (cudaMalloc(&base, bytes) != cudaSuccess) {
        cudaGetLastError();
        c->err = "swe_adjoint_gauge: out of device memory";
        return SWE_ERR_CUDA;
    }
    char *p = base;
    auto take = [&](size_t n) {
        char *q = p;
        p += (n + 255) / 256 * 256;
        return q;
    };
    for (int f = 0; f < 3; ++f) A.W[f] = (T *)take(A.fe * sizeof(T));
    A.gi = (int *)take(sizeof(int) * (n_gauges + 1));
    A.gj = (int *)take(sizeof(int) * (n_gauges + 1));
    A.obs = (double *)take(sizeof(double) * nobs);
    A.J = (double *)take(sizeof(double));
    A.speed = (unsigned long long *)take(2 * sizeof(unsigned long long));
    double *Jk = (double *)take((size_t)n_steps * sizeof(double));
    cudaStream_t st = c->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemsetAsync(Jk, 0, (size_t)n_steps * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.speed, 0, 2 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->flags, 0, sizeof(int), st);
    if (e == cudaSuccess && n_gauges > 0) {
        e = cudaMemcpyAsync(A.gi, gauge_i, sizeof(int) * n_gauges, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.gj, gauge_j, sizeof(int) * n_gauges, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.obs, h_obs, sizeof(double) * (nobs - 1), cudaMemcpyHostToDevice, st);
    }
    T *Un[3] = {static_cast<T *>(c->Un[0]), static_cast<T *>(c->Un[1]), static_cast<T *>(c->Un[2])};
    if (e == cudaSuccess) e = copy_state(A, A.W, Un);
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int k = 0; k < n_steps && e == cudaSuccess; ++k) {
        e = forward_step(A, A.W, A.W, false);
        if (e == cudaSuccess) {
            k_gauge<T><<<1, 32, 0, st>>>(A.W[0], static_cast<const T *>(c->B), c->pitch, A.gi,
                                         A.gj, A.ng, A.obs + (size_t)k * A.ng, nullptr, nullptr,
                                         Jk + k);
            ++c->launches;
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        k_sum_reverse<<<1, 32, 0, st>>>(Jk, n_steps, A.J);
        ++c->launches;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    double Jh = 0.0;
    int flags = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&Jh, A.J, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(base);
    if (e != cudaSuccess) {
        c->err = std::string("swe_adjoint_gauge: ") + cudaGetErrorString(e);
        return SWE_ERR_CUDA;
    }
    *J = Jh;
    if (ms) *ms = t;
    if (flags & FLAG_NONFINITE) {
        c->err = "non-finite state detected in GB300 adjoint";
        return SWE_ERR_NONFINITE;
    }
    return SWE_OK;
}

// The whole adjoint on a context whose state is of type T.
template <class T>
int run_adjoint(swe_ctx *c, int n_steps, double dt, int n_gauges, const int *gauge_i,
                const int *gauge_j, const double *h_obs, int n_snapshots, double *J,
                double *grad_h, double *grad_hu, double *grad_hv, double *grad_B, double *ms) {
    Adj<T> A;
    A.c = c;
    A.fe = c->field_elems;
    A.tape = n_snapshots == SWE_ADJ_TAPE_ALL;
    if (n_snapshots == SWE_ADJ_SEGMENTS) {
        A.seg_len = std::max(1, (int)std::lround(std::sqrt((double)n_steps)));
        A.nseg = (n_steps + A.seg_len - 1) / A.seg_len;
    }
    // snapshot slots: the binomial schedule's; tape: every state; segmented: the segment
    // starts plus the states of one taped segment
    A.S = A.tape ? n_steps
                 : (A.seg_len ? A.nseg + 1 + A.seg_len : std::min(n_snapshots, n_steps));
    const int tape_steps = A.tape ? n_steps : A.seg_len;  // steps of stage states kept
    A.ng = n_gauges;
    A.dt = dt;
    const size_t fb = A.fe * sizeof(T);
    auto rounded = [](size_t n) { return (n + 255) / 256 * 256; };
    // interface contributions in HBM: the FP64 two-pass reverse only
    const size_t cx_bytes = eta_state<T>() ? 0 : (size_t)NC * (c->p.Nx + 1) * c->p.Ny * sizeof(T);
    const size_t cy_bytes = eta_state<T>() ? 0 : (size_t)NC * c->p.Nx * (c->p.Ny + 1) * sizeof(T);
    const size_t wide = eta_state<T>() ? rounded(A.fe * sizeof(double)) : 0;  // output staging
    const size_t bytes = rounded((size_t)(A.S + 1) * 3 * fb) + 19 * rounded(fb) + 3 * rounded(A.fe) +
                         rounded(cx_bytes) + rounded(cy_bytes) + wide +
                         (tape_steps ? 2 * rounded((size_t)tape_steps * 3 * fb) +
                                           rounded((size_t)tape_steps * 3 * A.fe)
                                     : 0) +
                         2 * rounded(sizeof(int) * (n_gauges + 1)) +
                         rounded(sizeof(double) * ((size_t)n_steps * n_gauges + 1)) +
                         rounded(sizeof(double)) + rounded(2 * sizeof(unsigned long long));
    char *base = nullptr;
    if (cudaMalloc(&base, bytes) != cudaSuccess) {
        cudaGetLastError();
        c->err = "swe_adjoint_gauge: out of device memory for snapshots and adjoint state";
        return SWE_ERR_CUDA;
    }
    auto fail = [&](cudaError_t e) {
        cudaFree(base);
        c->err = std::string("swe_adjoint_gauge: ") + cudaGetErrorString(e);
        return SWE_ERR_CUDA;
    };
    char *p = base;
    auto take = [&](size_t n) {
        char *q = p;
        p += (n + 255) / 256 * 256;
        return q;
    };
    A.snap = (T *)take((size_t)(A.S + 1) * 3 * fb);
    for (int f = 0; f < 3; ++f) {
        A.W[f] = (T *)take(fb);
        A.Un1[f] = (T *)take(fb);
        A.lam[f] = (T *)take(fb);
        A.lamA[f] = (T *)take(fb);
        A.lamB[f] = (T *)take(fb);
        A.ln[f] = (T *)take(fb);
        A.mask[f] = (unsigned char *)take(A.fe);
    }
    A.gB = (T *)take(fb);
    A.cx = (T *)take(cx_bytes);
    A.cy = (T *)take(cy_bytes);
    double *widened = wide ? (double *)take(A.fe * sizeof(double)) : nullptr;
    if (tape_steps) {
        A.tU1 = (T *)take((size_t)tape_steps * 3 * fb);
        A.tU2 = (T *)take((size_t)tape_steps * 3 * fb);
        A.tmask = (unsigned char *)take((size_t)tape_steps * 3 * A.fe);
    }
    A.gi = (int *)take(sizeof(int) * (n_gauges + 1));
    A.gj = (int *)take(sizeof(int) * (n_gauges + 1));
    A.obs = (double *)take(sizeof(double) * ((size_t)n_steps * n_gauges + 1));
    A.J = (double *)take(sizeof(double));
    A.speed = (unsigned long long *)take(2 * sizeof(unsigned long long));
    cudaStream_t st = c->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaMemsetAsync(base, 0, bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->flags, 0, sizeof(int), st);
    if (e == cudaSuccess && n_gauges > 0) {
        e = cudaMemcpyAsync(A.gi, gauge_i, sizeof(int) * n_gauges, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.gj, gauge_j, sizeof(int) * n_gauges, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.obs, h_obs, sizeof(double) * (size_t)n_steps * n_gauges,
                                cudaMemcpyHostToDevice, st);
    }
    // slot 0 = U^0 (the context's state, left unchanged)
    T *Un[3] = {static_cast<T *>(c->Un[0]), static_cast<T *>(c->Un[1]), static_cast<T *>(c->Un[2])};
    if (e == cudaSuccess) e = copy_state(A, A.W, Un);
    if (e == cudaSuccess) e = store_slot(A, 0);
    if (e != cudaSuccess) return fail(e);
    if (!A.tape && !A.seg_len) build_schedule(A, n_steps, A.S);
    cudaEventRecord(e0, st);
    e = A.tape ? taped(A, n_steps)
               : (A.seg_len ? segmented(A, n_steps) : reverse(A, 0, n_steps, 0, A.S));
    cudaEventRecord(e1, st);
    if (e != cudaSuccess) return fail(e);
    double Jh = 0.0;
    int flags = 0;
    e = cudaMemcpyAsync(&Jh, A.J, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, st);
    const size_t row = (size_t)(c->p.Ny + 4) * sizeof(double), dp = (size_t)c->pitch * sizeof(double);
    double *outs[4] = {grad_h, grad_hu, grad_hv, grad_B};
    for (int f = 0; f < 4 && e == cudaSuccess; ++f) {
        const double *src;
        if (eta_state<T>()) {  // widen; dJ/dh0 = dJ/deta0, dJ/dB (h0 fixed) = gB + dJ/deta0
            const unsigned blocks = (unsigned)std::min<size_t>((A.fe + 255) / 256, 4096);
            const float *lam0 = reinterpret_cast<const float *>(A.lam[0]);
            if (f < 3)
                k_widen<<<blocks, 256, 0, st>>>(reinterpret_cast<const float *>(A.lam[f]), widened, A.fe);
            else
                k_grad_b_f32<<<blocks, 256, 0, st>>>(reinterpret_cast<const float *>(A.gB), lam0,
                                                     widened, A.fe);
            c->launches += 1;
            e = cudaGetLastError();
            src = widened;
        } else {
            src = reinterpret_cast<const double *>(f < 3 ? A.lam[f] : A.gB);
        }
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(outs[f], row, src, dp, row, (size_t)(c->p.Nx + 4),
                                  cudaMemcpyDeviceToHost, st);
        // the staging buffer is reused by the next field
        if (e == cudaSuccess && eta_state<T>()) e = cudaStreamSynchronize(st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return fail(e);
    cudaFree(base);
    *J = Jh;
    if (ms) *ms = t;
    if (flags & FLAG_NONFINITE) {
        c->err = "non-finite state detected in GB300 adjoint";
        return SWE_ERR_NONFINITE;
    }
    return SWE_OK;
}

}  // namespace
}  // namespace swe

using namespace swe;

extern "C" int swe_adjoint_gauge(swe_ctx *c, int n_steps, double dt, int n_gauges,
                                 const int *gauge_i, const int *gauge_j, const double *h_obs,
                                 int n_snapshots, double *J, double *grad_h, double *grad_hu,
                                 double *grad_hv, double *grad_B, double *ms) try {
    if (!c) return SWE_ERR_BAD_ARG;
    if (!c->uploaded || n_steps < 1 || !(dt > 0.0) ||
        n_gauges < 0 || (n_gauges > 0 && (!gauge_i || !gauge_j || !h_obs)) ||
        (n_snapshots < 0 && n_snapshots != SWE_ADJ_TAPE_ALL && n_snapshots != SWE_ADJ_SEGMENTS) ||
        !J ||
        (!grad_h + !grad_hu + !grad_hv + !grad_B) % 4 != 0) {
        c->err = "swe_adjoint_gauge: bad argument (needs an uploaded context)";
        return SWE_ERR_BAD_ARG;
    }
    if (c->p.x_halo_lo || c->p.x_halo_hi) {
        c->err = "swe_adjoint_gauge: not available on slab contexts";
        return SWE_ERR_UNSUPPORTED;
    }
    if (c->p.scheme != SWE_SCHEME_FUSED) {
        c->err = "swe_adjoint_gauge: the adjoint is of the fused scheme";
        return SWE_ERR_UNSUPPORTED;
    }
    for (int q = 0; q < n_gauges; ++q)
        if (gauge_i[q] < 0 || gauge_i[q] >= c->p.Nx || gauge_j[q] < 0 || gauge_j[q] >= c->p.Ny) {
            c->err = "swe_adjoint_gauge: gauge outside the interior";
            return SWE_ERR_BAD_ARG;
        }
    if (cudaSetDevice(c->p.device) != cudaSuccess) return SWE_ERR_CUDA;
    const bool f32 = c->p.precision == SWE_PRECISION_FP32_MIXED;
    if (!grad_h)  // every gradient pointer NULL: the objective alone
        return f32 ? run_objective<float>(c, n_steps, dt, n_gauges, gauge_i, gauge_j, h_obs, J, ms)
                   : run_objective<double>(c, n_steps, dt, n_gauges, gauge_i, gauge_j, h_obs, J, ms);
    if (f32)
        return run_adjoint<float>(c, n_steps, dt, n_gauges, gauge_i, gauge_j, h_obs, n_snapshots,
                                  J, grad_h, grad_hu, grad_hv, grad_B, ms);
    return run_adjoint<double>(c, n_steps, dt, n_gauges, gauge_i, gauge_j, h_obs, n_snapshots, J,
                               grad_h, grad_hu, grad_hv, grad_B, ms);
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}
