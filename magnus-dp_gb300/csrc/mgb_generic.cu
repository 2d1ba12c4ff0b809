// Generic engine kernels: any matrix dimension d, SpaceCurve, every rule.
//
//   k_chunk<MODE>  one CTA per (instance, chunk), persistent over a work list.
//       MODE_LOCAL : zero-carry pass, writes the chunk transfer Lambda^c.
//       MODE_CARRY : replays the chunk from its checkpoint pi^c and writes the
//                    reference-format carry P_k^(q)[i] = sum_j P_j[i] D_{k-j}^(q).
//       MODE_VJP   : replays the chunk from pi^c (tape of P_j), then runs the
//                    adjoint backwards from rho (cotangent on the chunk end
//                    state) and writes dA.
//     Level-major inside a chunk: a prefix pass (one thread per element,
//     sequential over the chunk's samples) alternates with a product pass
//     (flat over sample x element).  Chunk buffers live in a per-CTA slot of
//     global scratch memory.
//   k_scan         pi^{c+1} = Chen(Lambda^c, pi^c), FP64.
//   k_fin_fwd      D^(q), E, Omega and the output.
//   k_fin_vjp      cotangents tau_j on the totals T_j.
//   k_rscan        rho for every chunk (reverse scan).
//     One CTA per instance, or one warp per instance when n d^2 <= 256
//     (k_scan_w / k_rscan_w for the scans: step state in shared memory).
#include "mgb_common.cuh"
#include "mgb_kernels.h"

namespace mgb {

constexpr int NT = 256;

// ----------------------------------------------------------------------------
// chunk kernel
// ----------------------------------------------------------------------------
template <class T, int KIND, int RULE, int MODE>
__global__ void __launch_bounds__(NT) k_chunk(const InstDev* __restrict__ insts, const ChunkRef* __restrict__ work,
                                              int64_t nwork, T* __restrict__ scratch, int64_t slot_elems, int f64io) {
    using A_ = Alg<T, KIND>;
    T* slot = scratch + (int64_t)blockIdx.x * slot_elems;
    const bool f64 = f64io != 0;
    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        const ChunkRef wk = work[w];
        const InstDev& I = insts[wk.inst];
        const int c = wk.chunk;
        const int m = I.m, d = I.d, n = I.n;
        const int64_t b = (int64_t)c * I.K;
        const int64_t e = (b + I.K < I.S - 1) ? b + I.K : I.S - 1;
        const int Kp = (int)(e - b);
        const int L = Kp + 1;
        const bool riem0 = (RULE == R_RIEMANN) && c == 0;
        const int first = riem0 ? 0 : 1;
        const int64_t Lm = (int64_t)L * m;
        const int64_t nm = (int64_t)n * m;
        const RuleCoef<T> kc = rule_coef<T>(I);

        T* Ab = slot;             // [L][m]   A over the chunk
        T* tape = Ab + Lm;        // [n-1][L][m]  P_j over the chunk
        T* Wb = tape + (n - 1) * Lm;  // [L][m] level values W_{j+1}
        T* Gb = Wb + Lm;          // [L][m] cotangents on W_j
        T* Hb = Gb + Lm;          // [L][m] cotangents on P_j
        T* dAb = Hb + Lm;         // [L][m] dA accumulator

        for (int64_t idx = threadIdx.x; idx < Lm; idx += NT) {
            const int li = (int)(idx / m), el = (int)(idx - (int64_t)li * m);
            Ab[idx] = load_sample<T, KIND>(I.A, b + li, el, m, f64);
        }
        __syncthreads();

        const double* pic = I.pi + (int64_t)c * nm;
        // ---------------- forward over the chunk ----------------
        const T* F = Ab;
        for (int j = 1; j <= n; ++j) {
            T* Pj = tape + (int64_t)((j < n ? j : 1) - 1) * Lm;  // level n only needs its end value
            const bool keep = (j < n);
            for (int el = threadIdx.x; el < m; el += NT) {
                const double pij = (MODE == MODE_LOCAL || riem0) ? 0.0 : pic[(int64_t)(j - 1) * m + el];
                const Carry<T> cy = split_carry<T>(pij);
                FwdState<T> s;
                s.base = s.blo = T(0);
                s.f0 = F[el];
                s.f1 = s.f2 = s.f3 = T(0);
                if (!riem0 && keep) Pj[el] = add_carry(T(0), cy);
                for (int li = first; li <= Kp; ++li) {
                    const T P = fwd_step<T, RULE>(s, F[(int64_t)li * m + el], li, kc, cy);
                    if (keep) Pj[(int64_t)li * m + el] = P;
                }
                if (MODE == MODE_LOCAL) store_lam(I, (int64_t)c * nm + (int64_t)(j - 1) * m + el, s.base, s.blo);
            }
            __syncthreads();
            if (j < n) {
                for (int64_t idx = threadIdx.x; idx < Lm; idx += NT) {
                    const int li = (int)(idx / m), el = (int)(idx - (int64_t)li * m);
                    Wb[idx] = A_::mul(Ab + (int64_t)li * m, Pj + (int64_t)li * m, d, el);
                }
                __syncthreads();
                F = Wb;
            }
        }

        if (MODE == MODE_CARRY) {
            // carry[q][k-2][i] = sign_k * sum_{j=1}^{k-1} P_j[i] (x) D^(q)_{k-j}
            const int Q = I.Q;
            const int64_t S = I.S;
            const int lo = (c == 0) ? 0 : 1;
            const int64_t cnt = (int64_t)Q * (n - 1) * (L - lo) * m;
            for (int64_t idx = threadIdx.x; idx < cnt; idx += NT) {
                int64_t t = idx;
                const int el = (int)(t % m); t /= m;
                const int li = lo + (int)(t % (L - lo)); t /= (L - lo);
                const int k = 2 + (int)(t % (n - 1)); t /= (n - 1);
                const int q = (int)t;
                T acc = T(0);
                double sj = 1.0;
                for (int j = 1; j <= k - 1; ++j) {
                    sj *= I.sig;
                    const double* Dq = I.dq + ((int64_t)q * n + (k - j - 1)) * m;
                    acc += (T)sj * A_::mul(tape + (int64_t)(j - 1) * Lm + (int64_t)li * m, Dq, d, el);
                }
                if (KIND == KIND_SC && (k & 1)) acc = -acc;
                const int64_t off = (((int64_t)q * (n - 1) + (k - 2)) * S + (b + li)) * m + el;
                store_out<T>(I.carry, off, acc, f64);
            }
            __syncthreads();
        }

        if (MODE == MODE_VJP) {
            for (int64_t idx = threadIdx.x; idx < Lm; idx += NT) dAb[idx] = T(0);
            const double* rc = I.rho + (int64_t)c * nm;
            for (int j = n; j >= 1; --j) {
                if (j < n) {
                    const T* Pj = tape + (int64_t)(j - 1) * Lm;
                    for (int64_t idx = threadIdx.x; idx < Lm; idx += NT) {
                        const int li = (int)(idx / m), el = (int)(idx - (int64_t)li * m);
                        const T* g = Gb + (int64_t)li * m;
                        if (li >= first) Hb[idx] = A_::adjL(Ab + (int64_t)li * m, g, d, el);
                        dAb[idx] += A_::adjR(g, Pj + (int64_t)li * m, d, el);
                    }
                    __syncthreads();
                }
                for (int el = threadIdx.x; el < m; el += NT) {
                    const Carry<T> cy = split_carry<T>(rc[(int64_t)(j - 1) * m + el]);
                    RevState<T> s;
                    s.Rb = s.rlo = s.pend = s.R4l = s.R4 = s.H2 = s.H3 = T(0);
                    for (int li = Kp; li >= first; --li) {
                        const T H = (j < n) ? Hb[(int64_t)li * m + el] : T(0);
                        Gb[(int64_t)li * m + el] = rev_step<T, RULE>(s, H, li, kc, cy);
                    }
                    if (!riem0) Gb[el] = s.pend;
                }
                __syncthreads();
            }
            for (int64_t idx = threadIdx.x; idx < Lm; idx += NT) {
                const int li = (int)(idx / m), el = (int)(idx - (int64_t)li * m);
                if (RULE == R_RIEMANN && li == 0 && c > 0) continue;  // f_b unused by Riemann
                const T v = dAb[idx] + Gb[idx];
                const int64_t i = b + li;
                const bool shared = (li == 0 && c > 0) || (li == Kp && c < I.C - 1);
                int64_t off;
                if (KIND == KIND_SC) {
                    if (el == 0) continue;
                    off = i * 3 + (el - 1);
                } else {
                    off = i * (int64_t)m + el;
                }
                if (shared) atomic_add_out<T>(I.dA, off, v, f64);
                else store_out<T>(I.dA, off, v, f64);
            }
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------------------
// per-instance small math (FP64 storage, products in TS)
//
// G threads per instance: the whole CTA (NT) for large problems, one warp for
// small ones (n d^2 <= 256: 2x2 and 4x4 matrices, SpaceCurves), eight
// instances to a CTA.  These kernels are chains of short dependent steps
// (one per chunk in the scans), so packing the small instances one to a warp
// runs eight times as many chains at once.
// ----------------------------------------------------------------------------
template <int G>
struct Grp {
    int inst, t;
    __device__ __forceinline__ Grp() : inst((int)blockIdx.x * (NT / G) + (int)threadIdx.x / G), t((int)threadIdx.x % G) {}
    __device__ __forceinline__ void sync() const {
        if (G == NT) __syncthreads();
        else __syncwarp();
    }
};
template <class TS, int KIND, int G>
__global__ void __launch_bounds__(NT) k_scan(const InstDev* __restrict__ insts, int count) {
    using A_ = Alg<TS, KIND>;
    const Grp<G> grp;
    if (grp.inst >= count) return;
    const InstDev& I = insts[grp.inst];
    const int m = I.m, d = I.d, n = I.n;
    const int64_t nm = (int64_t)n * m;
    for (int64_t idx = grp.t; idx < nm; idx += G) I.pi[idx] = 0.0;
    grp.sync();
    for (int c = 0; c < I.C; ++c) {
        const double* pc = I.pi + (int64_t)c * nm;
        const double* lc = I.lam + (int64_t)c * nm;
        double* pn = I.pi + (int64_t)(c + 1) * nm;
        for (int64_t idx = grp.t; idx < nm; idx += G) {
            const int j = 1 + (int)(idx / m), el = (int)(idx % m);
            double v = pc[idx] + lc[idx];
            for (int mm = 1; mm < j; ++mm)
                v += (double)A_::mul(lc + (int64_t)(j - mm - 1) * m, pc + (int64_t)(mm - 1) * m, d, el);
            pn[idx] = v;
        }
        grp.sync();
    }
}

// D^(q)_k (k = 1..n), E_k, and (when out != nullptr) the op output.
template <class TS, int KIND, int G>
__global__ void __launch_bounds__(NT) k_fin_fwd(const InstDev* __restrict__ insts, int count, int f64io, int write_out) {
    using A_ = Alg<TS, KIND>;
    const Grp<G> grp;
    if (grp.inst >= count) return;
    const InstDev& I = insts[grp.inst];
    const int m = I.m, d = I.d, n = I.n, Q = I.Q;
    const int64_t nm = (int64_t)n * m;
    {
        const double* Tk = I.pi + (int64_t)I.C * nm;
        for (int64_t idx = grp.t; idx < nm; idx += G) {
            const int j = 1 + (int)(idx / m);
            I.tt[idx] = Tk[idx] * pow(I.sig, (double)j);
        }
        grp.sync();
    }
    const double* T_ = I.tt;
    for (int q = 0; q < Q; ++q) {
        double* Dq = I.dq + (int64_t)q * nm;
        const double s = I.glx[q] - 1.0;
        for (int el = grp.t; el < m; el += G) Dq[el] = (double)A_::one(d, el);
        grp.sync();
        for (int k = 2; k <= n; ++k) {
            for (int el = grp.t; el < m; el += G) {
                double v = T_[(int64_t)(k - 2) * m + el];  // T_{k-1} (x) D_1
                for (int j = 1; j <= k - 2; ++j)
                    v += (double)A_::mul(T_ + (int64_t)(j - 1) * m, Dq + (int64_t)(k - j - 1) * m, d, el);
                Dq[(int64_t)(k - 1) * m + el] = s * v;
            }
            grp.sync();
        }
    }
    for (int64_t idx = grp.t; idx < nm; idx += G) {
        double v = 0.0;
        for (int q = 0; q < Q; ++q) v += I.glw[q] * I.dq[(int64_t)q * nm + idx];
        I.ee[idx] = v;
    }
    grp.sync();
    // Omega_1 = T_1; Omega_k = sum_{j=1}^{k} T_j (x) E_{k-j+1}
    for (int64_t idx = grp.t; idx < nm; idx += G) {
        const int k = 1 + (int)(idx / m), el = (int)(idx % m);
        double v;
        if (k == 1) {
            v = T_[el];
        } else {
            v = 0.0;
            for (int j = 1; j <= k; ++j)
                v += (double)A_::mul(T_ + (int64_t)(j - 1) * m, I.ee + (int64_t)(k - j) * m, d, el);
        }
        if (KIND == KIND_SC && !(k & 1)) v = -v;
        I.ob[idx] = v;
    }
    grp.sync();
    if (!write_out) return;
    const bool f64 = f64io != 0;
    const int mo = (KIND == KIND_SC) ? 3 : m;
    const int off_el = (KIND == KIND_SC) ? 1 : 0;
    if (I.op == OP_MANY) {
        for (int64_t idx = grp.t; idx < (int64_t)n * mo; idx += G) {
            const int k = (int)(idx / mo), el = (int)(idx % mo);
            store_out<double>(I.out, idx, I.ob[(int64_t)k * m + el + off_el], f64);
        }
    } else {
        for (int el = grp.t; el < mo; el += G) {
            double v;
            if (I.op == OP_ONE) {
                v = I.ob[(int64_t)(n - 1) * m + el + off_el];
            } else {
                v = 0.0;
                for (int k = 0; k < n; ++k) v += I.ob[(int64_t)k * m + el + off_el];
            }
            store_out<double>(I.out, el, v, f64);
        }
    }
}

// tau_j = dL/dT_j from the output cotangent (E and D^(q) from k_fin_fwd).
template <class TS, int KIND, int G>
__global__ void __launch_bounds__(NT) k_fin_vjp(const InstDev* __restrict__ insts, int count, int f64io) {
    using A_ = Alg<TS, KIND>;
    const Grp<G> grp;
    if (grp.inst >= count) return;
    const InstDev& I = insts[grp.inst];
    const int m = I.m, d = I.d, n = I.n, Q = I.Q;
    const int64_t nm = (int64_t)n * m;
    const bool f64 = f64io != 0;
    const double* T_ = I.tt;
    // Omega-bar (SpaceCurve: padded, signed)
    for (int64_t idx = grp.t; idx < nm; idx += G) {
        const int k = 1 + (int)(idx / m), el = (int)(idx % m);
        double v = 0.0;
        int src_el = el;
        bool present = true;
        if (KIND == KIND_SC) {
            present = el != 0;
            src_el = el - 1;
        }
        const int mo = (KIND == KIND_SC) ? 3 : m;
        if (present) {
            if (I.op == OP_MANY) v = load_in<double>(I.cot, (int64_t)(k - 1) * mo + src_el, f64);
            else if (I.op == OP_SUM || k == n) v = load_in<double>(I.cot, src_el, f64);
        }
        if (KIND == KIND_SC && !(k & 1)) v = -v;
        I.ob[idx] = v;
        I.eb[idx] = 0.0;
    }
    grp.sync();
    // Ebar_m = sum_{k>=2, m=k-j+1>=2} adjL(T_j, Obar_k)
    for (int64_t idx = grp.t; idx < nm; idx += G) {
        const int mm = 1 + (int)(idx / m), el = (int)(idx % m);
        if (mm < 2) continue;
        double v = 0.0;
        for (int k = mm; k <= n; ++k) {
            const int j = k - mm + 1;
            v += (double)A_::adjL(T_ + (int64_t)(j - 1) * m, I.ob + (int64_t)(k - 1) * m, d, el);
        }
        I.eb[idx] = v;
    }
    // Tbar_j from the Omega assembly
    for (int64_t idx = grp.t; idx < nm; idx += G) {
        const int j = 1 + (int)(idx / m), el = (int)(idx % m);
        double v = (j == 1) ? I.ob[el] : 0.0;
        for (int k = (j > 2 ? j : 2); k <= n; ++k)
            v += (double)A_::adjR(I.ob + (int64_t)(k - 1) * m, I.ee + (int64_t)(k - j) * m, d, el);
        I.tau[idx] = v;
    }
    grp.sync();
    // back through D^(q)_k = s sum_{j<k} T_j D_{k-j}
    for (int q = 0; q < Q; ++q) {
        const double s = I.glx[q] - 1.0, wq = I.glw[q];
        const double* Dq = I.dq + (int64_t)q * nm;
        for (int64_t idx = grp.t; idx < nm; idx += G) I.db[idx] = wq * I.eb[idx];
        grp.sync();
        for (int k = n; k >= 2; --k) {
            const double* g = I.db + (int64_t)(k - 1) * m;  // s applied below
            for (int64_t idx = grp.t; idx < (int64_t)(k - 1) * m; idx += G) {
                const int j = 1 + (int)(idx / m), el = (int)(idx % m);
                I.tau[(int64_t)(j - 1) * m + el] += s * (double)A_::adjR(g, Dq + (int64_t)(k - j - 1) * m, d, el);
                if (k - j >= 2)
                    I.db[(int64_t)(k - j - 1) * m + el] += s * (double)A_::adjL(T_ + (int64_t)(j - 1) * m, g, d, el);
            }
            grp.sync();
        }
    }
    // cotangent on the kernels' unscaled totals: d/dT~_j = sig^j d/dT_j
    for (int64_t idx = grp.t; idx < nm; idx += G) {
        const int j = 1 + (int)(idx / m);
        I.tau[idx] *= pow(I.sig, (double)j);
    }
}

// rho[c] = cotangent on chunk c's end state; also zeroes the dA rows shared
// by two chunks (they are accumulated with atomics).
template <class TS, int KIND, int G>
__global__ void __launch_bounds__(NT) k_rscan(const InstDev* __restrict__ insts, int count, int f64io) {
    using A_ = Alg<TS, KIND>;
    const Grp<G> grp;
    if (grp.inst >= count) return;
    const InstDev& I = insts[grp.inst];
    const int m = I.m, d = I.d, n = I.n, C = I.C;
    const int64_t nm = (int64_t)n * m;
    const bool f64 = f64io != 0;
    double* last = I.rho + (int64_t)(C - 1) * nm;
    for (int64_t idx = grp.t; idx < nm; idx += G) last[idx] = I.tau[idx];
    grp.sync();
    for (int c = C - 1; c >= 1; --c) {
        const double* r = I.rho + (int64_t)c * nm;
        const double* lc = I.lam + (int64_t)c * nm;
        double* rn = I.rho + (int64_t)(c - 1) * nm;
        for (int64_t idx = grp.t; idx < nm; idx += G) {
            const int mm = 1 + (int)(idx / m), el = (int)(idx % m);
            double v = r[idx];
            for (int j = mm + 1; j <= n; ++j)
                v += (double)A_::adjL(lc + (int64_t)(j - mm - 1) * m, r + (int64_t)(j - 1) * m, d, el);
            rn[idx] = v;
        }
        grp.sync();
    }
    const int mo = (KIND == KIND_SC) ? 3 : m;
    for (int64_t idx = grp.t; idx < (int64_t)(C - 1) * mo; idx += G) {
        const int c = 1 + (int)(idx / mo), el = (int)(idx % mo);
        store_out<double>(I.dA, (int64_t)c * I.K * mo + el, 0.0, f64);
    }
}

// Warp-per-instance chunk scans (n d^2 <= 256): pi^c and Lambda^c of the
// step held in shared memory, Lambda^{c+1} loaded into registers while step
// c computes, so that a step costs shared-memory latency instead of an L2
// round trip per product operand.
constexpr int WMAX = 256, WEPL = WMAX / 32;

template <class TS, int KIND>
__global__ void __launch_bounds__(NT) k_scan_w(const InstDev* __restrict__ insts, int count) {
    using A_ = Alg<TS, KIND>;
    __shared__ double sp[NT / 32][WMAX], sl[NT / 32][WMAX];
    const Grp<32> grp;
    if (grp.inst >= count) return;
    const InstDev& I = insts[grp.inst];
    const int m = I.m, d = I.d, n = I.n, nm = n * m;
    double* P = sp[threadIdx.x / 32];
    double* L = sl[threadIdx.x / 32];
    double ln[WEPL];
#pragma unroll
    for (int e = 0; e < WEPL; ++e) {
        const int idx = grp.t + 32 * e;
        if (idx < nm) {
            P[idx] = 0.0;
            I.pi[idx] = 0.0;
            ln[e] = I.lam[idx];
        }
    }
    for (int c = 0; c < I.C; ++c) {
#pragma unroll
        for (int e = 0; e < WEPL; ++e) {
            const int idx = grp.t + 32 * e;
            if (idx < nm) L[idx] = ln[e];
        }
        __syncwarp();
        if (c + 1 < I.C) {
            const double* lx = I.lam + (int64_t)(c + 1) * nm;
#pragma unroll
            for (int e = 0; e < WEPL; ++e) {
                const int idx = grp.t + 32 * e;
                if (idx < nm) ln[e] = lx[idx];
            }
        }
        double v[WEPL];
#pragma unroll
        for (int e = 0; e < WEPL; ++e) {
            const int idx = grp.t + 32 * e;
            v[e] = 0.0;
            if (idx < nm) {
                const int j = 1 + idx / m, el = idx % m;
                double a = P[idx] + L[idx];
                for (int mm = 1; mm < j; ++mm) a += (double)A_::mul(L + (j - mm - 1) * m, P + (mm - 1) * m, d, el);
                v[e] = a;
            }
        }
        __syncwarp();
        double* pn = I.pi + (int64_t)(c + 1) * nm;
#pragma unroll
        for (int e = 0; e < WEPL; ++e) {
            const int idx = grp.t + 32 * e;
            if (idx < nm) {
                P[idx] = v[e];
                pn[idx] = v[e];
            }
        }
    }
}

// Warp-per-instance reverse scan (rho), the counterpart of k_scan_w.
template <class TS, int KIND>
__global__ void __launch_bounds__(NT) k_rscan_w(const InstDev* __restrict__ insts, int count, int f64io) {
    using A_ = Alg<TS, KIND>;
    __shared__ double sr[NT / 32][WMAX], sl[NT / 32][WMAX];
    const Grp<32> grp;
    if (grp.inst >= count) return;
    const InstDev& I = insts[grp.inst];
    const int m = I.m, d = I.d, n = I.n, nm = n * m, C = I.C;
    const bool f64 = f64io != 0;
    double* R = sr[threadIdx.x / 32];
    double* L = sl[threadIdx.x / 32];
    double ln[WEPL];
    double* last = I.rho + (int64_t)(C - 1) * nm;
#pragma unroll
    for (int e = 0; e < WEPL; ++e) {
        const int idx = grp.t + 32 * e;
        if (idx < nm) {
            const double t = I.tau[idx];
            R[idx] = t;
            last[idx] = t;
            if (C > 1) ln[e] = I.lam[(int64_t)(C - 1) * nm + idx];
        }
    }
    for (int c = C - 1; c >= 1; --c) {
#pragma unroll
        for (int e = 0; e < WEPL; ++e) {
            const int idx = grp.t + 32 * e;
            if (idx < nm) L[idx] = ln[e];
        }
        __syncwarp();
        if (c - 1 >= 1) {
            const double* lx = I.lam + (int64_t)(c - 1) * nm;
#pragma unroll
            for (int e = 0; e < WEPL; ++e) {
                const int idx = grp.t + 32 * e;
                if (idx < nm) ln[e] = lx[idx];
            }
        }
        double v[WEPL];
#pragma unroll
        for (int e = 0; e < WEPL; ++e) {
            const int idx = grp.t + 32 * e;
            v[e] = 0.0;
            if (idx < nm) {
                const int mm = 1 + idx / m, el = idx % m;
                double a = R[idx];
                for (int j = mm + 1; j <= n; ++j)
                    a += (double)A_::adjL(L + (j - mm - 1) * m, R + (j - 1) * m, d, el);
                v[e] = a;
            }
        }
        __syncwarp();
        double* rn = I.rho + (int64_t)(c - 1) * nm;
#pragma unroll
        for (int e = 0; e < WEPL; ++e) {
            const int idx = grp.t + 32 * e;
            if (idx < nm) {
                R[idx] = v[e];
                rn[idx] = v[e];
            }
        }
    }
    const int mo = (KIND == KIND_SC) ? 3 : m;
    for (int64_t idx = grp.t; idx < (int64_t)(C - 1) * mo; idx += 32) {
        const int c = 1 + (int)(idx / mo), el = (int)(idx % mo);
        store_out<double>(I.dA, (int64_t)c * I.K * mo + el, 0.0, f64);
    }
}

// ----------------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------------
template <class T, int KIND, int RULE>
static cudaError_t launch_chunk_t(int mode, const LaunchArgs& a) {
    dim3 grid((unsigned)a.grid), block(NT);
    T* scr = static_cast<T*>(a.scratch);
    if (mode == MODE_LOCAL)
        k_chunk<T, KIND, RULE, MODE_LOCAL><<<grid, block, 0, a.stream>>>(a.insts, a.work, a.nwork, scr, a.slot_elems, a.f64io);
    else if (mode == MODE_CARRY)
        k_chunk<T, KIND, RULE, MODE_CARRY><<<grid, block, 0, a.stream>>>(a.insts, a.work, a.nwork, scr, a.slot_elems, a.f64io);
    else
        k_chunk<T, KIND, RULE, MODE_VJP><<<grid, block, 0, a.stream>>>(a.insts, a.work, a.nwork, scr, a.slot_elems, a.f64io);
    return cudaGetLastError();
}

template <class T, int KIND>
static cudaError_t launch_chunk_k(int rule, int mode, const LaunchArgs& a) {
    switch (rule) {
        case R_BOOLE: return launch_chunk_t<T, KIND, R_BOOLE>(mode, a);
        case R_SIMPSON: return launch_chunk_t<T, KIND, R_SIMPSON>(mode, a);
        case R_TRAP: return launch_chunk_t<T, KIND, R_TRAP>(mode, a);
        default: return launch_chunk_t<T, KIND, R_RIEMANN>(mode, a);
    }
}

cudaError_t launch_generic_chunk(bool fp64, int kind, int rule, int mode, const LaunchArgs& a) {
    if (fp64) return kind == KIND_SC ? launch_chunk_k<double, KIND_SC>(rule, mode, a) : launch_chunk_k<double, KIND_MATRIX>(rule, mode, a);
    return kind == KIND_SC ? launch_chunk_k<float, KIND_SC>(rule, mode, a) : launch_chunk_k<float, KIND_MATRIX>(rule, mode, a);
}

template <class TS, int KIND, int G>
static cudaError_t launch_small_g(int which, const InstDev* insts, int count, int f64io, int write_out, cudaStream_t st) {
    constexpr int per = NT / G;  // instances per CTA
    dim3 grid((unsigned)((count + per - 1) / per)), block(NT);
    switch (which) {
        case SMALL_SCAN:
            if (G == 32) k_scan_w<TS, KIND><<<grid, block, 0, st>>>(insts, count);
            else k_scan<TS, KIND, G><<<grid, block, 0, st>>>(insts, count);
            break;
        case SMALL_FIN_FWD: k_fin_fwd<TS, KIND, G><<<grid, block, 0, st>>>(insts, count, f64io, write_out); break;
        case SMALL_FIN_VJP: k_fin_vjp<TS, KIND, G><<<grid, block, 0, st>>>(insts, count, f64io); break;
        default:
            if (G == 32) k_rscan_w<TS, KIND><<<grid, block, 0, st>>>(insts, count, f64io);
            else k_rscan<TS, KIND, G><<<grid, block, 0, st>>>(insts, count, f64io);
            break;
    }
    return cudaGetLastError();
}

template <class TS, int KIND>
static cudaError_t launch_small_k(int which, const InstDev* insts, int count, int f64io, int write_out, int64_t nm_max,
                                  cudaStream_t st) {
    if (nm_max <= 256) return launch_small_g<TS, KIND, 32>(which, insts, count, f64io, write_out, st);
    return launch_small_g<TS, KIND, NT>(which, insts, count, f64io, write_out, st);
}

cudaError_t launch_small(bool fp64, int kind, int which, const InstDev* insts, int count, int f64io, int write_out,
                         int64_t nm_max, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if (fp64) return kind == KIND_SC ? launch_small_k<double, KIND_SC>(which, insts, count, f64io, write_out, nm_max, st)
                                     : launch_small_k<double, KIND_MATRIX>(which, insts, count, f64io, write_out, nm_max, st);
    return kind == KIND_SC ? launch_small_k<float, KIND_SC>(which, insts, count, f64io, write_out, nm_max, st)
                           : launch_small_k<float, KIND_MATRIX>(which, insts, count, f64io, write_out, nm_max, st);
}

}  // namespace mgb
