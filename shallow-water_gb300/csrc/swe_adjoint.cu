// Discrete adjoint of the FP64 scheme with binomial checkpointing (C ABI:
// swe_adjoint_gauge in include/swe_gb300.h).
//
// Objective: J = sum over steps n = 1..N and gauge cells g of (h^n_g - h_obs^n_g)^2,
// fixed dt.  Gradients: dJ/dh^0, dJ/dhu^0, dJ/dhv^0 and dJ/dB (initial state held fixed).
//
// One adjoint step (transition k -> k+1, U^k in the work buffer):
//  1. recompute the three stages with clamp masks, U^(k+1) into a separate buffer;
//  2. add the gauge source 2 (h - h_obs) of step k+1 to lambda and accumulate J;
//  3. reverse stages 3, 2, 1 with k_adj_stage: per tile, recompute every interface whose
//     stencil touches the tile, apply its VJP (swe_adjoint_math.cuh) to the adjoint of the
//     divergence, and gather the contributions per cell (ghost slots folded onto the
//     interior cells they mirror, normal momentum negated at reflecting walls).  No
//     atomics: the result does not depend on scheduling.
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

#ifndef SWE_ADJ_MIN_BLOCKS
#define SWE_ADJ_MIN_BLOCKS 1  // resident CTAs per SM the register budget is sized for
#endif

constexpr int ATI = 8, ATJ = 32;
constexpr int ANT = (ATI + 3) * ATJ;       // one thread per x-face of the gather region
constexpr int SR = ATI + 6, SC = ATJ + 6;  // state tile, halo 3
constexpr int WR = ATI + 4, WC = ATJ + 4;  // divergence-adjoint tile, halo 2
constexpr int CR = ATI + 3, CC = ATJ + 3;  // contribution buffer (x: CR x ATJ, y: ATI x CC)

struct AdjSmem {
    double h[SR][SC], hu[SR][SC], hv[SR][SC], B[SR][SC], eta[SR][SC];
    double w[3][WR][WC];
    double C[14][CR][CC];  // per face: eta(4), qn(4), qt(4), bm, bp
};

struct AdjParams {
    const double *h, *hu, *hv, *B;       // stage source state, bathymetry
    const double *lo_h, *lo_hu, *lo_hv;  // adjoint of the stage output
    const unsigned char *mask;           // positivity clamps of this stage
    double *ls_h, *ls_hu, *ls_hv;        // adjoint of the stage source (written)
    double *ln_h, *ln_hu, *ln_hv;        // adjoint of U^n (stage 3 writes, 2 adds, 1 reads)
    double *gB;                          // dJ/dB (accumulated)
    int Nx, Ny;
    long long pitch;
    int bc;
    double inv_dx, inv_dy, g, dt;
};

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

template <int STAGE>
__global__ void __launch_bounds__(ANT, SWE_ADJ_MIN_BLOCKS) k_adj_stage(const AdjParams a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    AdjSmem &S = *reinterpret_cast<AdjSmem *>(smem_raw);
    const int tid = threadIdx.x;
    const int i0 = blockIdx.y * ATI, j0 = blockIdx.x * ATJ;
    const long long P = a.pitch;
    const double cs = STAGE == 1 ? 1.0 : (STAGE == 2 ? 0.25 : 2.0 / 3.0);

    for (int t = tid; t < SR * SC; t += ANT) {
        const int r = t / SC, c = t - (t / SC) * SC;
        const int ii = i0 - 3 + r, jj = j0 - 3 + c;
        bool fx, fy;
        const int mi = map_coord(ii, a.Nx, a.bc, fx), mj = map_coord(jj, a.Ny, a.bc, fy);
        const long long k = (long long)(mi + NG) * P + (mj + NG);
        const double h = a.h[k], hu = a.hu[k], hv = a.hv[k];
        const int bi = clamp_int(ii + NG, 0, a.Nx + 3), bj = clamp_int(jj + NG, 0, a.Ny + 3);
        const double b = a.B[(long long)bi * P + bj];
        S.h[r][c] = h;
        S.hu[r][c] = fx ? -hu : hu;
        S.hv[r][c] = fy ? -hv : hv;
        S.B[r][c] = b;
        S.eta[r][c] = h + b;
    }
    for (int t = tid; t < WR * WC; t += ANT) {
        const int r = t / WC, c = t - (t / WC) * WC;
        const int ii = i0 - 2 + r, jj = j0 - 2 + c;
        double w0 = 0.0, w1 = 0.0, w2 = 0.0;
        if (ii >= 0 && ii < a.Nx && jj >= 0 && jj < a.Ny) {
            const long long k = (long long)(ii + NG) * P + (jj + NG);
            if (!a.mask[k]) {
                const double f = cs * a.dt;
                w0 = f * a.lo_h[k];
                w1 = f * a.lo_hu[k];
                w2 = f * a.lo_hv[k];
            }
        }
        S.w[0][r][c] = w0;
        S.w[1][r][c] = w1;
        S.w[2][r][c] = w2;
    }
    __syncthreads();

    // ---- x-faces f in [i0-2, i0+ATI]: one per thread ----
    {
        const int fr = tid / ATJ, col = tid - (tid / ATJ) * ATJ;
        const int f = i0 - 2 + fr, jj = j0 + col;
        adj::FaceIn<double> ad;
        for (int q = 0; q < 4; ++q) ad.e[q] = ad.n[q] = ad.t[q] = 0.0;
        ad.bm = ad.bp = 0.0;
        if (f >= -1 && f <= a.Nx - 1 && jj < a.Ny) {
            adj::FaceIn<double> in;
            for (int q = 0; q < 4; ++q) {
                in.e[q] = S.eta[fr + q][col + 3];
                in.n[q] = S.hu[fr + q][col + 3];
                in.t[q] = S.hv[fr + q][col + 3];
            }
            in.bm = S.B[fr + 1][col + 3];
            in.bp = S.B[fr + 2][col + 3];
            adj::FaceOut<double> d;
            d.fh = a.inv_dx * (S.w[0][fr + 1][col + 2] - S.w[0][fr][col + 2]);
            d.fqt = a.inv_dx * (S.w[2][fr + 1][col + 2] - S.w[2][fr][col + 2]);
            d.fqn_m = -a.inv_dx * S.w[1][fr][col + 2];
            d.fqn_p = a.inv_dx * S.w[1][fr + 1][col + 2];
            adj::face_vjp(in, a.g, EPS, d, ad);
        }
        for (int q = 0; q < 4; ++q) {
            S.C[q][fr][col] = ad.e[q];
            S.C[4 + q][fr][col] = ad.n[q];
            S.C[8 + q][fr][col] = ad.t[q];
        }
        S.C[12][fr][col] = ad.bm;
        S.C[13][fr][col] = ad.bp;
    }
    __syncthreads();

    const int ty = tid / ATJ, tx = tid - (tid / ATJ) * ATJ;
    const int ci = i0 + ty, cj = j0 + tx;
    const bool own = tid < ATI * ATJ && ci < a.Nx && cj < a.Ny;
    double acc_h = 0.0, acc_hu = 0.0, acc_hv = 0.0, acc_B = 0.0;
    if (own) {
        int v[5];
        bool fl[5];
        const int nv = virtual_coords(ci, a.Nx, a.bc, v, fl);
        for (int q = 0; q < nv; ++q) {
            for (int k = 0; k < 4; ++k) {
                const int f = v[q] + 1 - k;  // face whose stencil slot k is row v
                const int fr = f - i0 + 2;
                if (f < -1 || f > a.Nx - 1 || fr < 0 || fr >= CR) continue;
                const double ce = S.C[k][fr][tx], cn = S.C[4 + k][fr][tx];
                acc_h += ce;
                acc_B += ce;
                acc_hu += fl[q] ? -cn : cn;
                acc_hv += S.C[8 + k][fr][tx];
            }
            const int fm = v[q], fp = v[q] - 1;  // faces with row v as minus / plus cell
            if (fm >= -1 && fm <= a.Nx - 1 && fm - i0 + 2 >= 0 && fm - i0 + 2 < CR)
                acc_B += S.C[12][fm - i0 + 2][tx];
            if (fp >= -1 && fp <= a.Nx - 1 && fp - i0 + 2 >= 0 && fp - i0 + 2 < CR)
                acc_B += S.C[13][fp - i0 + 2][tx];
        }
    }
    __syncthreads();

    // ---- y-faces f in [j0-2, j0+ATJ] for the tile rows ----
    if (tid < ATI * CC) {
        const int row = tid / CC, gc = tid - (tid / CC) * CC;
        const int f = j0 - 2 + gc, ii = i0 + row;
        adj::FaceIn<double> ad;
        for (int q = 0; q < 4; ++q) ad.e[q] = ad.n[q] = ad.t[q] = 0.0;
        ad.bm = ad.bp = 0.0;
        if (f >= -1 && f <= a.Ny - 1 && ii < a.Nx) {
            adj::FaceIn<double> in;
            for (int q = 0; q < 4; ++q) {
                in.e[q] = S.eta[row + 3][gc + q];
                in.n[q] = S.hv[row + 3][gc + q];
                in.t[q] = S.hu[row + 3][gc + q];
            }
            in.bm = S.B[row + 3][gc + 1];
            in.bp = S.B[row + 3][gc + 2];
            adj::FaceOut<double> d;
            d.fh = a.inv_dy * (S.w[0][row + 2][gc + 1] - S.w[0][row + 2][gc]);
            d.fqt = a.inv_dy * (S.w[1][row + 2][gc + 1] - S.w[1][row + 2][gc]);
            d.fqn_m = -a.inv_dy * S.w[2][row + 2][gc];
            d.fqn_p = a.inv_dy * S.w[2][row + 2][gc + 1];
            adj::face_vjp(in, a.g, EPS, d, ad);
        }
        for (int q = 0; q < 4; ++q) {
            S.C[q][row][gc] = ad.e[q];
            S.C[4 + q][row][gc] = ad.n[q];
            S.C[8 + q][row][gc] = ad.t[q];
        }
        S.C[12][row][gc] = ad.bm;
        S.C[13][row][gc] = ad.bp;
    }
    __syncthreads();

    if (!own) return;
    {
        int v[5];
        bool fl[5];
        const int nv = virtual_coords(cj, a.Ny, a.bc, v, fl);
        for (int q = 0; q < nv; ++q) {
            for (int k = 0; k < 4; ++k) {
                const int f = v[q] + 1 - k;
                const int gc = f - j0 + 2;
                if (f < -1 || f > a.Ny - 1 || gc < 0 || gc >= CC) continue;
                const double ce = S.C[k][ty][gc], cn = S.C[4 + k][ty][gc];
                acc_h += ce;
                acc_B += ce;
                acc_hv += fl[q] ? -cn : cn;
                acc_hu += S.C[8 + k][ty][gc];
            }
            const int fm = v[q], fp = v[q] - 1;
            if (fm >= -1 && fm <= a.Ny - 1 && fm - j0 + 2 >= 0 && fm - j0 + 2 < CC)
                acc_B += S.C[12][ty][fm - j0 + 2];
            if (fp >= -1 && fp <= a.Ny - 1 && fp - j0 + 2 >= 0 && fp - j0 + 2 < CC)
                acc_B += S.C[13][ty][fp - j0 + 2];
        }
    }
    const long long k = (long long)(ci + NG) * P + (cj + NG);
    const bool m = a.mask[k];
    const double l0 = m ? 0.0 : a.lo_h[k], l1 = m ? 0.0 : a.lo_hu[k], l2 = m ? 0.0 : a.lo_hv[k];
    double o0 = acc_h + cs * l0, o1 = acc_hu + cs * l1, o2 = acc_hv + cs * l2;
    if (STAGE == 3) {
        a.ln_h[k] = l0 / 3.0;
        a.ln_hu[k] = l1 / 3.0;
        a.ln_hv[k] = l2 / 3.0;
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

// One forward step W -> out (out may be W); masks optional.
cudaError_t forward_step(Adj &A, double *const *W, double *const *out, bool masks) {
    swe_ctx *c = A.c;
    StageParams sp = fwd_params(A);
    double *U1[3] = {(double *)c->U1[0], (double *)c->U1[1], (double *)c->U1[2]};
    double *U2[3] = {(double *)c->U2[0], (double *)c->U2[1], (double *)c->U2[2]};
    sp.hn = W[0]; sp.hun = W[1]; sp.hvn = W[2];
    sp.hs = W[0]; sp.hus = W[1]; sp.hvs = W[2];
    sp.ho = U1[0]; sp.huo = U1[1]; sp.hvo = U1[2];
    sp.mask = masks ? A.mask[0] : nullptr;
    ACK(launch_stage_f64(1, sp, c->stream));
    sp.hs = U1[0]; sp.hus = U1[1]; sp.hvs = U1[2];
    sp.ho = U2[0]; sp.huo = U2[1]; sp.hvo = U2[2];
    sp.mask = masks ? A.mask[1] : nullptr;
    ACK(launch_stage_f64(2, sp, c->stream));
    sp.hs = U2[0]; sp.hus = U2[1]; sp.hvs = U2[2];
    sp.ho = out[0]; sp.huo = out[1]; sp.hvo = out[2];
    sp.mask = masks ? A.mask[2] : nullptr;
    ACK(launch_stage_f64(3, sp, c->stream));
    c->launches += 3;
    ++A.fwd_steps;
    return cudaSuccess;
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
    const dim3 grid((c->p.Ny + ATJ - 1) / ATJ, (c->p.Nx + ATI - 1) / ATI);
    const size_t smem = sizeof(AdjSmem);
    switch (stage) {
        case 1: k_adj_stage<1><<<grid, ANT, smem, c->stream>>>(p); break;
        case 2: k_adj_stage<2><<<grid, ANT, smem, c->stream>>>(p); break;
        default: k_adj_stage<3><<<grid, ANT, smem, c->stream>>>(p); break;
    }
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

bool adj_attr_set = false;

}  // namespace
}  // namespace swe

using namespace swe;

extern "C" int swe_adjoint_gauge(swe_ctx *c, int n_steps, double dt, int n_gauges,
                                 const int *gauge_i, const int *gauge_j, const double *h_obs,
                                 int n_snapshots, double *J, double *grad_h, double *grad_hu,
                                 double *grad_hv, double *grad_B, double *ms) {
    if (!c) return SWE_ERR_BAD_ARG;
    if (!c->uploaded || c->p.precision != SWE_PRECISION_FP64 || n_steps < 1 || !(dt > 0.0) ||
        n_gauges < 0 || (n_gauges > 0 && (!gauge_i || !gauge_j || !h_obs)) || n_snapshots < 0 ||
        !J || !grad_h || !grad_hu || !grad_hv || !grad_B) {
        c->err = "swe_adjoint_gauge: bad argument (needs an uploaded FP64 context)";
        return SWE_ERR_BAD_ARG;
    }
    for (int q = 0; q < n_gauges; ++q)
        if (gauge_i[q] < 0 || gauge_i[q] >= c->p.Nx || gauge_j[q] < 0 || gauge_j[q] >= c->p.Ny) {
            c->err = "swe_adjoint_gauge: gauge outside the interior";
            return SWE_ERR_BAD_ARG;
        }
    if (cudaSetDevice(c->p.device) != cudaSuccess) return SWE_ERR_CUDA;
    if (!adj_attr_set) {
        for (auto k : {k_adj_stage<1>, k_adj_stage<2>, k_adj_stage<3>})
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(AdjSmem)) != cudaSuccess) {
                c->err = "swe_adjoint_gauge: cannot opt in to the adjoint kernel's shared memory";
                return SWE_ERR_CUDA;
            }
        adj_attr_set = true;
    }
    Adj A;
    A.c = c;
    A.fe = c->field_elems;
    A.S = std::min(n_snapshots, n_steps);
    A.ng = n_gauges;
    A.dt = dt;
    const size_t fb = A.fe * sizeof(double);
    auto rounded = [](size_t n) { return (n + 255) / 256 * 256; };
    const size_t bytes = rounded((size_t)(A.S + 1) * 3 * fb) + 19 * rounded(fb) + 3 * rounded(A.fe) +
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
    build_schedule(A, n_steps, A.S);
    cudaEventRecord(e0, st);
    e = reverse(A, 0, n_steps, 0, A.S);
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
