// Discrete adjoint of the FP64 scheme with binomial checkpointing (C ABI:
// swe_adjoint_gauge in include/swe_gb300.h).
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
#include <cstdint>
#include <cstring>
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

struct AdjParams {
    const double *h, *hu, *hv, *B;       // stage source state, bathymetry
    const double *lo_h, *lo_hu, *lo_hv;  // adjoint of the stage output
    const unsigned char *mask;           // positivity clamps of this stage
    double *ls_h, *ls_hu, *ls_hv;        // adjoint of the stage source (written)
    double *ln_h, *ln_hu, *ln_hv;        // adjoint of U^n (stage 3 writes, 2 adds, 1 reads)
    double *gB;                          // dJ/dB (accumulated)
    double *cx, *cy;                     // interface contributions, NC planes each
    long long px, py;                    // plane sizes: (Nx + 1) * Ny, Nx * (Ny + 1)
    int Nx, Ny;
    long long pitch;
    int bc;
    double inv_dx, inv_dy, g, dt;
};

// Adjoint of the divergence at interior cell (i, j): cs * dt * lo, zero where the stage
// clamped the depth (its output did not depend on the fluxes there) and outside.
template <int STAGE>
__device__ __forceinline__ void w_at(const AdjParams &a, int i, int j, double w[3]) {
    constexpr double cs = STAGE == 1 ? 1.0 : (STAGE == 2 ? 0.25 : 2.0 / 3.0);
    w[0] = w[1] = w[2] = 0.0;
    if (i < 0 || i >= a.Nx || j < 0 || j >= a.Ny) return;
    const long long k = (long long)(i + NG) * a.pitch + (j + NG);
    if (a.mask[k]) return;
    const double f = cs * a.dt;
    w[0] = f * a.lo_h[k];
    w[1] = f * a.lo_hu[k];
    w[2] = f * a.lo_hv[k];
}

// One interface per thread.  DIR 0: x-interface f in [-1, Nx - 1] between rows f and
// f + 1 at column j; DIR 1: y-interface f in [-1, Ny - 1] between columns f and f + 1 at
// row i.  The stencil is staged exactly as the forward kernel stages it: the state of
// ghost cells from the mirrored (reflecting, normal momentum negated) or clamped
// (transmissive) interior cell, B where it lies, ghosts included.
template <int STAGE, int DIR>
__global__ void __launch_bounds__(AFT) k_adj_faces(const AdjParams a) {
    const int t = blockIdx.x * AFT + threadIdx.x;
    const int along = DIR == 0 ? a.Ny : a.Ny + 1;  // contiguous index range
    if (t >= along) return;
    const int f = DIR == 0 ? (int)blockIdx.y - 1 : t - 1;  // interface index
    const int o = DIR == 0 ? t : (int)blockIdx.y;          // the other coordinate
    const long long P = a.pitch;
    adj::FaceIn<double> in;
    for (int q = 0; q < 4; ++q) {
        const int c = f - 1 + q;  // stencil cell along the normal
        bool fl;
        const int m = map_coord(c, DIR == 0 ? a.Nx : a.Ny, a.bc, fl);
        const long long ks = DIR == 0 ? (long long)(m + NG) * P + (o + NG)
                                      : (long long)(o + NG) * P + (m + NG);
        const int cb = clamp_int(c + NG, 0, (DIR == 0 ? a.Nx : a.Ny) + 3);
        const long long kb = DIR == 0 ? (long long)cb * P + (o + NG) : (long long)(o + NG) * P + cb;
        const double b = a.B[kb];
        const double qn = DIR == 0 ? a.hu[ks] : a.hv[ks];
        in.e[q] = a.h[ks] + b;
        in.n[q] = fl ? -qn : qn;
        in.t[q] = DIR == 0 ? a.hv[ks] : a.hu[ks];
        if (q == 1) in.bm = b;
        if (q == 2) in.bp = b;
    }
    double wm[3], wp[3];
    if (DIR == 0) {
        w_at<STAGE>(a, f, o, wm);
        w_at<STAGE>(a, f + 1, o, wp);
    } else {
        w_at<STAGE>(a, o, f, wm);
        w_at<STAGE>(a, o, f + 1, wp);
    }
    const double inv = DIR == 0 ? a.inv_dx : a.inv_dy;
    const int n = DIR == 0 ? 1 : 2, tg = DIR == 0 ? 2 : 1;  // normal / tangential field
    adj::FaceOut<double> d;
    d.fh = inv * (wp[0] - wm[0]);
    d.fqt = inv * (wp[tg] - wm[tg]);
    d.fqn_m = -inv * wm[n];
    d.fqn_p = inv * wp[n];
    adj::FaceIn<double> ad;
    adj::face_vjp(in, a.g, EPS, d, ad);
    double *C = DIR == 0 ? a.cx : a.cy;
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
template <int DIR>
__device__ __forceinline__ void gather_dir(const AdjParams &a, int ca, int other, double &acc_h,
                                           double &acc_qn, double &acc_qt, double &acc_B) {
    const int N = DIR == 0 ? a.Nx : a.Ny;
    const double *C = DIR == 0 ? a.cx : a.cy;
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
            const double ce = C[k * pl + x], cn = C[(4 + k) * pl + x];
            acc_h += ce;
            acc_B += ce;
            acc_qn += fl[q] ? -cn : cn;
            acc_qt += C[(8 + k) * pl + x];
        }
        const int fm = v[q], fp = v[q] - 1;  // interfaces with cell v as minus / plus side
        if (fm >= -1 && fm <= N - 1) acc_B += C[12 * pl + at(fm)];
        if (fp >= -1 && fp <= N - 1) acc_B += C[13 * pl + at(fp)];
    }
}

// Per interior cell: adjoint of the stage source and of U^n, and dJ/dB.
template <int STAGE>
__global__ void __launch_bounds__(AGT) k_adj_gather(const AdjParams a) {
    const int cj = blockIdx.x * AGT + threadIdx.x, ci = blockIdx.y;
    if (cj >= a.Ny) return;
    constexpr double cs = STAGE == 1 ? 1.0 : (STAGE == 2 ? 0.25 : 2.0 / 3.0);
    double acc_h = 0.0, acc_hu = 0.0, acc_hv = 0.0, acc_B = 0.0;
    gather_dir<0>(a, ci, cj, acc_h, acc_hu, acc_hv, acc_B);
    gather_dir<1>(a, cj, ci, acc_h, acc_hv, acc_hu, acc_B);
    const long long k = (long long)(ci + NG) * a.pitch + (cj + NG);
    const bool m = a.mask[k];
    const double l0 = m ? 0.0 : a.lo_h[k], l1 = m ? 0.0 : a.lo_hu[k], l2 = m ? 0.0 : a.lo_hv[k];
    double o0 = acc_h + cs * l0, o1 = acc_hu + cs * l1, o2 = acc_hv + cs * l2;
    if (STAGE == 3) {  // the forward's (1.0 / 3.0) * U^n
        a.ln_h[k] = (1.0 / 3.0) * l0;
        a.ln_hu[k] = (1.0 / 3.0) * l1;
        a.ln_hv[k] = (1.0 / 3.0) * l2;
    } else if (STAGE == 2) {
        a.ln_h[k] += 0.75 * l0;
        a.ln_hu[k] += 0.75 * l1;
        a.ln_hv[k] += 0.75 * l2;
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
__global__ void k_gauge(const double *h, long long P, const int *gi, const int *gj, int ng,
                        const double *obs, double *lam_h, double *J) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int q = 0; q < ng; ++q) {
        const long long k = (long long)(gi[q] + NG) * P + (gj[q] + NG);
        const double r = h[k] - obs[q];
        s += r * r;
        lam_h[k] += 2.0 * r;
    }
    *J += s;
}

struct Adj {
    swe_ctx *c;
    size_t fe;  // elements per field
    double *snap;
    int S;
    double *W[3], *Un1[3], *lam[3], *lamA[3], *lamB[3], *ln[3], *gB;
    double *cx, *cy;  // interface contributions of the stage being reversed
    bool tape = false;              // every state and every step's stage states kept
    double *tU1 = nullptr, *tU2 = nullptr;  // tape: U^(1), U^(2) of step k at 3 k fields
    unsigned char *tmask = nullptr;         // tape: clamp masks of step k at 3 k fields
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

StageParams fwd_params(const Adj &A) {
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
    sp.cfl_min_dxdy = c->cfl_min_dxdy;
    sp.dt_fixed = A.dt;
    sp.speed = A.speed;  // scratch slots: the context's adaptive-dt slots stay untouched
    sp.slot_read = 0;
    sp.slot_write = 1;
    sp.flags = c->flags;
    return sp;
}

// One forward step W -> out (out may be W) with the stage states in U1, U2 and the
// clamp masks in mk[0..2] (null: not kept).
cudaError_t forward_step_into(Adj &A, double *const *W, double *const *out, double *const *U1,
                              double *const *U2, unsigned char *const *mk) {
    swe_ctx *c = A.c;
    StageParams sp = fwd_params(A);
    sp.hn = W[0]; sp.hun = W[1]; sp.hvn = W[2];
    sp.hs = W[0]; sp.hus = W[1]; sp.hvs = W[2];
    sp.ho = U1[0]; sp.huo = U1[1]; sp.hvo = U1[2];
    sp.mask = mk[0];
    ACK(launch_stage_f64(1, sp, nullptr, c->stream));
    sp.hs = U1[0]; sp.hus = U1[1]; sp.hvs = U1[2];
    sp.ho = U2[0]; sp.huo = U2[1]; sp.hvo = U2[2];
    sp.mask = mk[1];
    ACK(launch_stage_f64(2, sp, nullptr, c->stream));
    sp.hs = U2[0]; sp.hus = U2[1]; sp.hvs = U2[2];
    sp.ho = out[0]; sp.huo = out[1]; sp.hvo = out[2];
    sp.mask = mk[2];
    ACK(launch_stage_f64(3, sp, nullptr, c->stream));
    c->launches += 3;
    ++A.fwd_steps;
    return cudaSuccess;
}

// One forward step W -> out through the context's stage buffers; masks optional.
cudaError_t forward_step(Adj &A, double *const *W, double *const *out, bool masks) {
    swe_ctx *c = A.c;
    double *U1[3] = {(double *)c->U1[0], (double *)c->U1[1], (double *)c->U1[2]};
    double *U2[3] = {(double *)c->U2[0], (double *)c->U2[1], (double *)c->U2[2]};
    unsigned char *none[3] = {nullptr, nullptr, nullptr};
    return forward_step_into(A, W, out, U1, U2, masks ? A.mask : none);
}

cudaError_t launch_adj(Adj &A, int stage, double *const *state, double *const *lo,
                       const unsigned char *mask, double *const *ls) {
    swe_ctx *c = A.c;
    AdjParams p{};
    p.h = state[0]; p.hu = state[1]; p.hv = state[2];
    p.B = (const double *)c->B;
    p.lo_h = lo[0]; p.lo_hu = lo[1]; p.lo_hv = lo[2];
    p.mask = mask;
    p.ls_h = ls[0]; p.ls_hu = ls[1]; p.ls_hv = ls[2];
    p.ln_h = A.ln[0]; p.ln_hu = A.ln[1]; p.ln_hv = A.ln[2];
    p.gB = A.gB;
    p.Nx = c->p.Nx;
    p.Ny = c->p.Ny;
    p.pitch = c->pitch;
    p.bc = c->p.bc;
    p.inv_dx = c->inv_dx;
    p.inv_dy = c->inv_dy;
    p.g = c->p.g;
    p.dt = A.dt;
    p.cx = A.cx;
    p.cy = A.cy;
    p.px = (long long)(c->p.Nx + 1) * c->p.Ny;
    p.py = (long long)c->p.Nx * (c->p.Ny + 1);
    const dim3 gx((c->p.Ny + AFT - 1) / AFT, c->p.Nx + 1), gy((c->p.Ny + 1 + AFT - 1) / AFT, c->p.Nx);
    const dim3 gg((c->p.Ny + AGT - 1) / AGT, c->p.Nx);
    switch (stage) {
        case 1:
            k_adj_faces<1, 0><<<gx, AFT, 0, c->stream>>>(p);
            k_adj_faces<1, 1><<<gy, AFT, 0, c->stream>>>(p);
            k_adj_gather<1><<<gg, AGT, 0, c->stream>>>(p);
            break;
        case 2:
            k_adj_faces<2, 0><<<gx, AFT, 0, c->stream>>>(p);
            k_adj_faces<2, 1><<<gy, AFT, 0, c->stream>>>(p);
            k_adj_gather<2><<<gg, AGT, 0, c->stream>>>(p);
            break;
        default:
            k_adj_faces<3, 0><<<gx, AFT, 0, c->stream>>>(p);
            k_adj_faces<3, 1><<<gy, AFT, 0, c->stream>>>(p);
            k_adj_gather<3><<<gg, AGT, 0, c->stream>>>(p);
            break;
    }
    c->launches += 2;
    ++c->launches;
    return cudaGetLastError();
}

// Adjoint of step k (W holds U^k; lam holds the adjoint of U^(k+1) before its source).
cudaError_t adjoint_step(Adj &A, int k) {
    swe_ctx *c = A.c;
    ACK(forward_step(A, A.W, A.Un1, true));
    double *U1[3] = {(double *)c->U1[0], (double *)c->U1[1], (double *)c->U1[2]};
    double *U2[3] = {(double *)c->U2[0], (double *)c->U2[1], (double *)c->U2[2]};
    k_gauge<<<1, 32, 0, c->stream>>>(A.Un1[0], c->pitch, A.gi, A.gj, A.ng,
                                     A.obs + (size_t)k * A.ng, A.lam[0], A.J);
    ++c->launches;
    ACK(cudaGetLastError());
    ACK(launch_adj(A, 3, U2, A.lam, A.mask[2], A.lamA));
    ACK(launch_adj(A, 2, U1, A.lamA, A.mask[1], A.lamB));
    ACK(launch_adj(A, 1, A.W, A.lamB, A.mask[0], A.lam));
    return cudaSuccess;
}

cudaError_t copy_state(Adj &A, double *const *dst, double *const *src) {
    for (int f = 0; f < 3; ++f)
        ACK(cudaMemcpyAsync(dst[f], src[f], A.fe * sizeof(double), cudaMemcpyDeviceToDevice,
                            A.c->stream));
    return cudaSuccess;
}

double *slot_field(Adj &A, int slot, int f) { return A.snap + ((size_t)slot * 3 + f) * A.fe; }

cudaError_t load_slot(Adj &A, int slot) {
    double *src[3] = {slot_field(A, slot, 0), slot_field(A, slot, 1), slot_field(A, slot, 2)};
    return copy_state(A, A.W, src);
}

cudaError_t store_slot(Adj &A, int slot) {
    double *dst[3] = {slot_field(A, slot, 0), slot_field(A, slot, 1), slot_field(A, slot, 2)};
    return copy_state(A, dst, A.W);
}

double *tape_field(double *base, Adj &A, int k, int f) { return base + ((size_t)k * 3 + f) * A.fe; }

// Tape mode: one forward sweep keeps U^k in slot k and the stage states and clamp masks
// of step k in the tape; the reverse sweep then recomputes nothing.
cudaError_t taped(Adj &A, int n) {
    swe_ctx *c = A.c;
    for (int k = 0; k < n; ++k) {
        double *W[3], *out[3], *U1[3], *U2[3];
        unsigned char *mk[3];
        for (int f = 0; f < 3; ++f) {
            W[f] = slot_field(A, k, f);
            out[f] = slot_field(A, k + 1, f);
            U1[f] = tape_field(A.tU1, A, k, f);
            U2[f] = tape_field(A.tU2, A, k, f);
            mk[f] = A.tmask + ((size_t)k * 3 + f) * A.fe;
        }
        ACK(forward_step_into(A, W, out, U1, U2, mk));
    }
    for (int k = n - 1; k >= 0; --k) {
        double *Wk[3], *U1[3], *U2[3];
        const unsigned char *mk[3];
        for (int f = 0; f < 3; ++f) {
            Wk[f] = slot_field(A, k, f);
            U1[f] = tape_field(A.tU1, A, k, f);
            U2[f] = tape_field(A.tU2, A, k, f);
            mk[f] = A.tmask + ((size_t)k * 3 + f) * A.fe;
        }
        k_gauge<<<1, 32, 0, c->stream>>>(slot_field(A, k + 1, 0), c->pitch, A.gi, A.gj, A.ng,
                                         A.obs + (size_t)k * A.ng, A.lam[0], A.J);
        ++c->launches;
        ACK(cudaGetLastError());
        ACK(launch_adj(A, 3, U2, A.lam, mk[2], A.lamA));
        ACK(launch_adj(A, 2, U1, A.lamA, mk[1], A.lamB));
        ACK(launch_adj(A, 1, Wk, A.lamB, mk[0], A.lam));
    }
    return cudaSuccess;
}

// Adjoint of steps [l, l+n) with U^l in `slot` and s free snapshot slots.
cudaError_t reverse(Adj &A, int l, int n, int slot, int s) {
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
void build_schedule(Adj &A, int N, int S) {
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

}  // namespace
}  // namespace swe

using namespace swe;

extern "C" int swe_adjoint_gauge(swe_ctx *c, int n_steps, double dt, int n_gauges,
                                 const int *gauge_i, const int *gauge_j, const double *h_obs,
                                 int n_snapshots, double *J, double *grad_h, double *grad_hu,
                                 double *grad_hv, double *grad_B, double *ms) {
    if (!c) return SWE_ERR_BAD_ARG;
    if (!c->uploaded || c->p.precision != SWE_PRECISION_FP64 || n_steps < 1 || !(dt > 0.0) ||
        n_gauges < 0 || (n_gauges > 0 && (!gauge_i || !gauge_j || !h_obs)) ||
        (n_snapshots < 0 && n_snapshots != SWE_ADJ_TAPE_ALL) ||
        !J || !grad_h || !grad_hu || !grad_hv || !grad_B) {
        c->err = "swe_adjoint_gauge: bad argument (needs an uploaded FP64 context)";
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
    Adj A;
    A.c = c;
    A.fe = c->field_elems;
    A.tape = n_snapshots == SWE_ADJ_TAPE_ALL;
    A.S = A.tape ? n_steps : std::min(n_snapshots, n_steps);
    A.ng = n_gauges;
    A.dt = dt;
    const size_t fb = A.fe * sizeof(double);
    auto rounded = [](size_t n) { return (n + 255) / 256 * 256; };
    const size_t cx_bytes = (size_t)NC * (c->p.Nx + 1) * c->p.Ny * sizeof(double);
    const size_t cy_bytes = (size_t)NC * c->p.Nx * (c->p.Ny + 1) * sizeof(double);
    const size_t bytes = rounded((size_t)(A.S + 1) * 3 * fb) + 19 * rounded(fb) + 3 * rounded(A.fe) +
                         rounded(cx_bytes) + rounded(cy_bytes) +
                         (A.tape ? 2 * rounded((size_t)n_steps * 3 * fb) +
                                       rounded((size_t)n_steps * 3 * A.fe)
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
    A.snap = (double *)take((size_t)(A.S + 1) * 3 * fb);
    for (int f = 0; f < 3; ++f) {
        A.W[f] = (double *)take(fb);
        A.Un1[f] = (double *)take(fb);
        A.lam[f] = (double *)take(fb);
        A.lamA[f] = (double *)take(fb);
        A.lamB[f] = (double *)take(fb);
        A.ln[f] = (double *)take(fb);
        A.mask[f] = (unsigned char *)take(A.fe);
    }
    A.gB = (double *)take(fb);
    A.cx = (double *)take(cx_bytes);
    A.cy = (double *)take(cy_bytes);
    if (A.tape) {
        A.tU1 = (double *)take((size_t)n_steps * 3 * fb);
        A.tU2 = (double *)take((size_t)n_steps * 3 * fb);
        A.tmask = (unsigned char *)take((size_t)n_steps * 3 * A.fe);
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
    double *Un[3] = {(double *)c->Un[0], (double *)c->Un[1], (double *)c->Un[2]};
    if (e == cudaSuccess) e = copy_state(A, A.W, Un);
    if (e == cudaSuccess) e = store_slot(A, 0);
    if (e != cudaSuccess) return fail(e);
    if (!A.tape) build_schedule(A, n_steps, A.S);
    cudaEventRecord(e0, st);
    e = A.tape ? taped(A, n_steps) : reverse(A, 0, n_steps, 0, A.S);
    cudaEventRecord(e1, st);
    if (e != cudaSuccess) return fail(e);
    double Jh = 0.0;
    int flags = 0;
    e = cudaMemcpyAsync(&Jh, A.J, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, st);
    const size_t row = (size_t)(c->p.Ny + 4) * sizeof(double), dp = (size_t)c->pitch * sizeof(double);
    double *outs[4] = {grad_h, grad_hu, grad_hv, grad_B};
    double *srcs[4] = {A.lam[0], A.lam[1], A.lam[2], A.gB};
    for (int f = 0; f < 4 && e == cudaSuccess; ++f)
        e = cudaMemcpy2DAsync(outs[f], row, srcs[f], dp, row, (size_t)(c->p.Nx + 4),
                              cudaMemcpyDeviceToHost, st);
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
