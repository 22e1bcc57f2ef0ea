// The round-robin dataflow LU-SGS sweeps of the flow equations as device
// functions: the binary64 form (one cell per warp) and the binary32 form (two
// cells of one level per warp).  k_fp64.cu launches them alone; k_sst.cu
// launches them beside the turbulence equations' sweep in one cooperative
// grid, the flow on blocks [0, B) and the turbulence on the rest, each block
// numbered within its part (bid).  vnp_out (may be null) receives, per
// (cell, face slot) with a contributing neighbour j, Vn(W_j + dW_j): the
// updated normal velocity the turbulence sweep needs for the same slot (the
// binary32 form also its exact change Vn(W_j + dW_j) - Vn(W_j)).
#pragma once

#include "case.hpp"
#include "fv_kernels.cuh"

namespace cfdgb {

// "increment not yet computed" marker of the dataflow LU-SGS sweep: a
// signalling NaN, a bit pattern arithmetic never produces
constexpr unsigned long long kSentinel = 0x7ff4c0ffee5eed11ULL;
constexpr unsigned kSentinelF = 0x7fa0c0deu;  // a signalling binary32 NaN
constexpr long long kSpinLimit = 1LL << 22;

__device__ __forceinline__ bool is_sentinel(double x) {
    return (unsigned long long)__double_as_longlong(x) == kSentinel;
}
__device__ __forceinline__ bool is_sentinel_f(float x) { return __float_as_uint(x) == kSentinelF; }
__device__ __forceinline__ bool ready_f4(const float4& v) {
    return !is_sentinel_f(v.x) && !is_sentinel_f(v.y) && !is_sentinel_f(v.z) && !is_sentinel_f(v.w);
}

template <bool FWD, bool PF>
__device__ __forceinline__ void sweep_flow_body(int bid, int B, int nc, const int* __restrict__ order,
                                                    const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                    const d4* __restrict__ fg0, const d4* __restrict__ W,
                                                    const double* __restrict__ swfc, const double* __restrict__ swra,
                                                    const d4* __restrict__ R, const double* __restrict__ D,
                                                    const double* __restrict__ invD, d4* dW1, d4* dW,
                                                    unsigned* err, int poll_ns, double* vnp_out) {
    // One warp per cell.  Lanes 0..15: (face slot s, equation m); lanes 16..31
    // mirror them and only help with the divide (v = w3/w0 beside u = w2/w0).
    const double GM1 = 1.4 - 1.0;
    const int lane = threadIdx.x & 31;
    const int hv = lane >> 4;
    const int s = (lane >> 2) & 3, m = lane & 3;
    const int warp = threadIdx.x >> 5;
    const int NW = blockDim.x >> 5;
    d4* dst = FWD ? dW1 : dW;
    // Position p = block + B*q goes to block p % B and warp (q + block) % NW:
    // consecutive positions (one level's cells) land on different SMs and, as
    // the warp index rotates with the block, on different SM sub-partitions
    // (whose FP64 pipes are separate).  Each warp visits its positions in
    // increasing order: q = q0, q0 + NW, q0 + 2*NW, ...
    const int q0 = ((warp - (int)(bid % NW)) % NW + NW) % NW;
    // PF: the inputs of a position that do not depend on a neighbour's
    // increment (cell, face slot, neighbour, its W, the face, the per-step
    // SolveDF constants and the cell's own term) are loaded one position ahead,
    // while the warp waits for the current position's neighbour, so their
    // chain of dependent loads stays off the sweep's critical path; it costs
    // registers (fewer resident warps), which wide levels may need more, so the
    // autotuner tries both.
    struct In {
        int i, j;
        int4 cf;
        bool use, left;
        double w0[4];
        d4 g;
        double fc, rA, own, dinv;
    };
    auto load = [&](long long p, In& x) {
        x.i = order[p];
        x.cf = cface[x.i];
        const int code = s == 0 ? x.cf.x : s == 1 ? x.cf.y : s == 2 ? x.cf.z : x.cf.w;
        x.use = false;
        x.left = false;
        x.j = 0;
        int f = 0;
        if (code != 0) {
            f = code_face(code);
            x.left = code > 0;
            int2 e = lr[f];
            x.j = x.left ? e.y : e.x;
            x.use = FWD ? (x.j >= 0 && x.j < x.i) : (x.j > x.i);
        }
        // this cell's own inputs of the final update: R_i (forward) or dW1_i (backward), and D_i
        x.own = 0.0;
        x.dinv = 1.0;
        if (lane < 4) {
            x.own = FWD ? (&R[x.i].x)[m] : (&dW1[x.i].x)[m];
            x.dinv = D[x.i];
        }
        // lanes without a contributing neighbour compute on harmless values and
        // are masked at the end, so the arithmetic is issued once per warp
        x.w0[0] = 1.0; x.w0[1] = 1.0; x.w0[2] = 0.0; x.w0[3] = 0.0;
        x.g = d4{0.0, 0.0, 0.0, 0.0};
        x.fc = 0.0;
        x.rA = 0.0;
        if (x.use) {
            to_arr(ld4(W + x.j), x.w0);
            x.g = fg0[f];
            x.fc = swfc[(size_t)x.i * 16 + s * 4 + m];
            x.rA = swra[(size_t)x.i * 4 + s];
        }
    };
    long long p = (long long)bid + (long long)B * q0;
    if (p >= nc) return;
    In cur, nxt;
    load(p, cur);
    for (;;) {
        const long long pn = p + (long long)B * NW;
        const bool more = pn < nc;
        if (PF && more) load(pn, nxt);
        double dw[4] = {0.0, 0.0, 0.0, 0.0};
        if (cur.use) {
            // the neighbour's increment is final once none of its four words is
            // the sentinel (each aligned 8-byte word is written exactly once)
            const double2* q = reinterpret_cast<const double2*>(dst + cur.j);
            double2 a, b;
            long long it = 0;
            while (true) {
                a = __ldcv(q);
                b = __ldcv(q + 1);
                if (!is_sentinel(a.x) && !is_sentinel(a.y) && !is_sentinel(b.x) && !is_sentinel(b.y)) break;
                if (++it > kSpinLimit) {
                    atomicOr(err, ERR_TIMEOUT);
                    break;
                }
                if (poll_ns > 0) __nanosleep(poll_ns);
            }
            dw[0] = a.x; dw[1] = a.y; dw[2] = b.x; dw[3] = b.y;
        }
        __syncwarp();  // reconverge before the arithmetic
        double wp[4];
#pragma unroll
        for (int k = 0; k < 4; k++) wp[k] = cur.w0[k] + dw[k];
        // one divide per half-warp, exchanged
        const double quo = (hv ? wp[3] : wp[2]) / wp[0];
        const double u = __shfl_sync(0xffffffffu, quo, lane & 15);
        const double v = __shfl_sync(0xffffffffu, quo, (lane & 15) | 16);
        const d4 g = cur.g;
        double vn = dot2(u, v, g.x, g.y);
        // Vn(W_j + dW_j) on this face is the turbulence sweep's input for the same (cell, slot)
        if (vnp_out && cur.use && hv == 0 && m == 0) __stcg(vnp_out + (size_t)cur.i * 4 + s, vn);
        double pr = GM1 * (wp[1] - 0.5 * wp[0] * sq2(u, v));
        double fcp = m == 0 ? wp[0] * vn : m == 1 ? (wp[1] + pr) * vn : m == 2 ? wp[2] * vn + pr * g.x
                                                                               : wp[3] * vn + pr * g.y;
        double dwm = m == 0 ? dw[0] : m == 1 ? dw[1] : m == 2 ? dw[2] : dw[3];
        double dfc = cur.left ? (fcp - cur.fc) : (cur.fc - fcp);
        double df = 0.5 * (dfc - cur.rA * dwm) * g.z;
        const double DF = cur.use ? df : 0.0;
        // ordered sum over the 4 face slots (lanes m, m+4, m+8, m+12)
        double v0 = __shfl_sync(0xffffffffu, DF, m);
        double v1 = __shfl_sync(0xffffffffu, DF, 4 + m);
        double v2 = __shfl_sync(0xffffffffu, DF, 8 + m);
        double v3 = __shfl_sync(0xffffffffu, DF, 12 + m);
        double dF = 0.0;
        if (cur.cf.x != 0) dF += v0;
        if (cur.cf.y != 0) dF += v1;
        if (cur.cf.z != 0) dF += v2;
        if (cur.cf.w != 0) dF += v3;
        double res = 0.0;
        if (lane < 4) {
            if (FWD) res = (-cur.own - dF) / cur.dinv;
            else res = cur.own - dF / cur.dinv;
        }
        double r1 = __shfl_sync(0xffffffffu, res, 1);
        double r2 = __shfl_sync(0xffffffffu, res, 2);
        double r3 = __shfl_sync(0xffffffffu, res, 3);
        if (lane == 0) {
            double2* o = reinterpret_cast<double2*>(dst + cur.i);
            __stcg(o, make_double2(res, r1));
            __stcg(o + 1, make_double2(r2, r3));
        }
        if (!more) break;
        if (!PF) load(pn, nxt);
        cur = nxt;
        p = pn;
    }
}

template <bool FWD, bool IND, bool PF>
__device__ __forceinline__ void sweep_flow32_body(int bid, int B, int npos, const int* __restrict__ order2,
                                                      const int4* __restrict__ cface, const int2* __restrict__ lr,
                                                      const float4* __restrict__ fg0f, const float4* __restrict__ Wf,
                                                      const float* __restrict__ swraf,
                                                      const d4* __restrict__ R, const double* __restrict__ invD,
                                                      d4* dW1, d4* dW, float4* dW1f, float4* dWf, unsigned* err,
                                                      int poll_ns, float2* vnp_out) {
    const float GM1 = 1.4f - 1.0f;
    const int lane = threadIdx.x & 31;
    const int h = lane >> 4, base = lane & 16;
    const int s = (lane >> 2) & 3, m = lane & 3;
    const int warp = threadIdx.x >> 5;
    const int NW = blockDim.x >> 5;
    d4* dst = FWD ? dW1 : dW;
    float4* dstf = FWD ? dW1f : dWf;
    const int npairs = npos >> 1;
    // IND: the two half-warps synchronise and exchange only among themselves,
    // so a cell whose neighbours are ready does not wait for its pair partner
    const unsigned mask = IND ? (h ? 0xffff0000u : 0x0000ffffu) : 0xffffffffu;
    const int q0 = ((warp - (int)(bid % NW)) % NW + NW) % NW;
    // The inputs of a pair position that do not depend on a neighbour's
    // increment - its cells, slots and neighbours, the neighbour's binary32
    // state with the base values of its flux (formed before the wait, so that
    // only the difference terms remain on the dependence chain), r_A and the
    // cell's own term - are loaded and formed one position ahead (PF), while
    // the warp waits for the current position's neighbours.
    struct In {
        int i, j;
        bool active, use, left;
        int4 cf;
        float4 w0, g;
        float rA, u, v, vv, p, vn;
        double own, dinv;
        float ownf, dinvf;  // their binary32 roundings, formed here rather than on the dependence chain
    };
    auto load = [&](long long P, In& x) {
        x.i = order2[2 * P + h];
        x.active = x.i >= 0;
        x.cf = x.active ? cface[x.i] : make_int4(0, 0, 0, 0);
        const int code = s == 0 ? x.cf.x : s == 1 ? x.cf.y : s == 2 ? x.cf.z : x.cf.w;
        x.use = false;
        x.left = false;
        x.j = 0;
        int f = 0;
        if (code != 0) {
            f = code_face(code);
            x.left = code > 0;
            int2 e = lr[f];
            x.j = x.left ? e.y : e.x;
            x.use = FWD ? (x.j >= 0 && x.j < x.i) : (x.j > x.i);
        }
        x.own = 0.0;
        x.dinv = 1.0;
        if (x.active && s == 0) {
            x.own = FWD ? (&R[x.i].x)[m] : (&dW1[x.i].x)[m];
            x.dinv = invD[x.i];
        }
        x.ownf = (float)x.own;
        x.dinvf = (float)x.dinv;
        x.w0 = make_float4(1.f, 1.f, 0.f, 0.f);
        x.g = make_float4(0.f, 0.f, 0.f, 0.f);
        x.rA = x.u = x.v = x.vv = x.p = x.vn = 0.f;
        if (x.use) {
            x.w0 = Wf[x.j];
            x.g = fg0f[f];
            x.rA = swraf[(size_t)x.i * 4 + s];
            x.u = x.w0.z / x.w0.x;
            x.v = x.w0.w / x.w0.x;
            x.vv = x.u * x.u + x.v * x.v;
            x.p = GM1 * (x.w0.y - 0.5f * x.w0.x * x.vv);
            x.vn = x.u * x.g.x + x.v * x.g.y;
        }
    };
    long long P = (long long)bid + (long long)B * q0;  // pair index, same mapping as k_sweep_flow
    if (P >= npairs) return;
    In cur, nxt;
    load(P, cur);
    for (;;) {
        const long long Pn = P + (long long)B * NW;
        const bool more = Pn < npairs;
        if (PF && more) load(Pn, nxt);
        float4 dw = make_float4(0.f, 0.f, 0.f, 0.f);
        if (cur.use) {
            const float4* qf = (FWD ? dW1f : dWf) + cur.j;
            long long it = 0;
            while (true) {
                dw = __ldcv(qf);
                if (ready_f4(dw)) break;
                if (++it > kSpinLimit) {
                    atomicOr(err, ERR_TIMEOUT);
                    break;
                }
                if (poll_ns > 0) __nanosleep(poll_ns);
            }
        }
        __syncwarp(mask);
        // F(W + dW) - F(W) as an exact difference: every term is a product of a
        // difference with base or updated values, so its relative error does
        // not grow as dW shrinks below W's binary32 resolution (subtracting two
        // binary32 fluxes would leave a noise of ~1e-7 |F| that stalls the
        // mixed form's convergence near a 5e-5 residual fall).
        const float rho = cur.w0.x, E = cur.w0.y, mx = cur.w0.z, my = cur.w0.w;
        const float u = cur.u, v = cur.v, vv = cur.vv, p = cur.p, vn = cur.vn;
        const float4 g = cur.g;
        const float d0 = dw.x, d1 = dw.y, d2 = dw.z, d3 = dw.w;
        const float rp = 1.f / (rho + d0);
        const float du = (d2 - u * d0) * rp, dv = (d3 - v * d0) * rp;
        const float dq = du * (u + u + du) + dv * (v + v + dv);
        const float dp = GM1 * (d1 - 0.5f * (d0 * (vv + dq) + rho * dq));
        const float dvn = du * g.x + dv * g.y;
        const float vnp = vn + dvn;
        // Vn(W_j + dW_j) on this face and its exact change are the turbulence sweep's input for the same
        // (cell, slot)
        if (vnp_out && cur.use && m == 0) __stcg(vnp_out + (size_t)cur.i * 4 + s, make_float2(vnp, dvn));
        const float dfm = m == 0 ? d2 * g.x + d3 * g.y
                        : m == 1 ? (d1 + dp) * vnp + (E + p) * dvn
                        : m == 2 ? d2 * vnp + mx * dvn + dp * g.x
                                 : d3 * vnp + my * dvn + dp * g.y;
        float dwm = m == 0 ? dw.x : m == 1 ? dw.y : m == 2 ? dw.z : dw.w;
        float dfc = cur.left ? dfm : -dfm;
        float DF = cur.use ? 0.5f * (dfc - cur.rA * dwm) * g.z : 0.f;
        float v0 = __shfl_sync(mask, DF, base + m);
        float v1 = __shfl_sync(mask, DF, base + 4 + m);
        float v2 = __shfl_sync(mask, DF, base + 8 + m);
        float v3 = __shfl_sync(mask, DF, base + 12 + m);
        float dF = 0.f;
        if (cur.cf.x != 0) dF += v0;
        if (cur.cf.y != 0) dF += v1;
        if (cur.cf.z != 0) dF += v2;
        if (cur.cf.w != 0) dF += v3;
        // The binary32 copy that the next levels wait for is computed and
        // published first, in binary32; the binary64 increment (used only by
        // the backward sweep and the update, after this launch) follows off
        // the critical path.
        const float resf = FWD ? (-cur.ownf - dF) * cur.dinvf : cur.ownf - dF * cur.dinvf;
        // one 16-byte store (measured faster than each lane storing its own word: readers then
        // saw partly written records and polled again)
        float f1 = __shfl_sync(mask, resf, base + 1);
        float f2 = __shfl_sync(mask, resf, base + 2);
        float f3 = __shfl_sync(mask, resf, base + 3);
        if (cur.active && (lane & 15) == 0) __stcg(dstf + cur.i, make_float4(resf, f1, f2, f3));
        double res = 0.0;
        if (s == 0) res = FWD ? (-cur.own - (double)dF) * cur.dinv : cur.own - (double)dF * cur.dinv;
        double r1 = __shfl_sync(mask, res, base + 1);
        double r2 = __shfl_sync(mask, res, base + 2);
        double r3 = __shfl_sync(mask, res, base + 3);
        if (cur.active && (lane & 15) == 0) {
            double2* o = reinterpret_cast<double2*>(dst + cur.i);
            __stcg(o, make_double2(res, r1));
            __stcg(o + 1, make_double2(r2, r3));
        }
        if (!more) break;
        if (!PF) load(Pn, nxt);
        cur = nxt;
        P = Pn;
    }
}

}  // namespace cfdgb
