// Batched FFTs of lines held in shared memory: mixed-radix (3/2/4/8)
// Stockham passes, and for the common FP32 lengths the two-step form below.
//
// The lines of one thread block live in shared memory, line l at a + l*ls,
// elements contiguous.  Each stage reads radix-r butterfly inputs with stride
// L/r, applies the twiddles w^(t*k), does the r-point DFT in registers and
// writes the outputs in autosorted (Stockham) order into the other buffer, so
// no bit reversal is needed.  Twiddles come from a per-block table in
// shared memory built from tw[m] = exp(-2*pi*i*m/L) (load_twiddles: one block
// of entries per stage, read by consecutive lanes); the inverse uses their
// conjugates and leaves the 1/L normalisation to the caller.
#pragma once
#include "sc_common.cuh"

namespace ocsc {

template <typename C, bool INV>
__device__ __forceinline__ void dft2(C& a, C& b) {
    C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <typename C, bool INV>
__device__ __forceinline__ void dft4(C& a0, C& a1, C& a2, C& a3) {
    C t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = csub(a1, a3);
    t3 = INV ? cmul_pi(t3) : cmul_mi(t3);
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

// 3-point DFT: y_k = sum_t a_t w^(t k), w = exp(-2 pi i / 3) (forward) or its
// conjugate (inverse): y0 = a + (b + c), y1,2 = a - (b + c)/2 -/+ i (sqrt(3)/2)(b - c)
template <typename R, bool INV>
__device__ __forceinline__ void dft3(Cx<R>& a, Cx<R>& b, Cx<R>& c) {
    const R s = INV ? (R)-0.86602540378443864676 : (R)0.86602540378443864676;
    const Cx<R> t = cadd(b, c), d = csub(b, c);
    const Cx<R> m = cx<R>(a.x - (R)0.5 * t.x, a.y - (R)0.5 * t.y);
    const Cx<R> r = cx<R>(s * d.y, -s * d.x);  // -i s d
    a = cadd(a, t);
    b = cadd(m, r);
    c = csub(m, r);
}

template <typename R, bool INV>
__device__ __forceinline__ void dft8(Cx<R>* v) {
    Cx<R> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    Cx<R> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<Cx<R>, INV>(e0, e1, e2, e3);
    dft4<Cx<R>, INV>(o0, o1, o2, o3);
    const R h = (R)0.70710678118654752440;
    if (!INV) {  // w = exp(-i*pi/4)
        o1 = cx<R>((o1.x + o1.y) * h, (o1.y - o1.x) * h);
        o2 = cmul_mi(o2);
        o3 = cx<R>((o3.y - o3.x) * h, (-o3.x - o3.y) * h);
    } else {     // w = exp(+i*pi/4)
        o1 = cx<R>((o1.x - o1.y) * h, (o1.x + o1.y) * h);
        o2 = cmul_pi(o2);
        o3 = cx<R>((-o3.x - o3.y) * h, (o3.x - o3.y) * h);
    }
    v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
}

// tw: the stage twiddle table of load_twiddles; the stage's block starts at
// Ns - (the first stage's radix)
template <typename R, bool INV, int RAD>
__device__ __forceinline__ void stockham_stage(const Cx<R>* __restrict__ a, Cx<R>* __restrict__ b,
                                               int L, int ls, int nl, int Ns, const Cx<R>* tw, int tw_off) {
    const int nb = L / RAD;
    const int total = nb * nl;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int line = idx / nb;
        const int j = idx - line * nb;
        const Cx<R>* src = a + line * ls;
        Cx<R>* dst = b + line * ls;
        const int k = j % Ns;
        Cx<R> v[RAD];
#pragma unroll
        for (int t = 0; t < RAD; ++t) v[t] = src[j + t * nb];
        if (Ns > 1) {
#pragma unroll
            for (int t = 1; t < RAD; ++t) {
                Cx<R> w = tw[tw_off + (t - 1) * Ns + k];
                if (INV) w.y = -w.y;
                v[t] = cmul(v[t], w);
            }
        }
        if (RAD == 2) dft2<Cx<R>, INV>(v[0], v[1]);
        else if (RAD == 3) dft3<R, INV>(v[0], v[1], v[2]);
        else if (RAD == 4) dft4<Cx<R>, INV>(v[0], v[1], v[2], v[3]);
        else dft8<R, INV>(v);
        const int out = (j - k) * RAD + k;
#pragma unroll
        for (int t = 0; t < RAD; ++t) dst[out + t * Ns] = v[t];
    }
}

// The same stages with the line length known at compile time: the radix of
// each stage, the butterfly count and the twiddle stride are constants, so
// the index arithmetic reduces to shifts, masks and multiplications.  The
// plan is the one of make_radix_plan (for lengths 3 * 2^k one radix-3 stage,
// then radix 8 while it divides, then 4, then 2) and the arithmetic is that
// of stockham_stage, so results are identical.
constexpr int plan_radix(int L, int s) {
    int rem = L, st = 0;
    if (rem % 3 == 0) {
        if (st == s) return 3;
        rem /= 3;
        ++st;
    }
    while (rem % 8 == 0 && rem > 1) {
        if (st == s) return 8;
        rem /= 8;
        ++st;
    }
    while (rem % 4 == 0 && rem > 1) {
        if (st == s) return 4;
        rem /= 4;
        ++st;
    }
    while (rem % 2 == 0 && rem > 1) {
        if (st == s) return 2;
        rem /= 2;
        ++st;
    }
    return 0;
}

// Intermediate stages keep element i of a line at a padded position: the
// Stockham output index of the early stages strides by RAD elements per
// thread, which in the plain layout puts 8 or more threads of a warp on the
// same bank.  One pad element per 16 (lines of 128 points and more) spreads
// those strides over all banks and keeps the 16 lanes of a half-warp that
// read consecutive elements on 16 distinct bank pairs; with one pad per 8 the
// half-warp's 16 elements spanned 17 slots and its first and last lane met on
// one bank (a shared-memory model of the stages: 11% fewer wavefronts at 128
// points, 10% at 512).  Shorter lines keep one pad per 8, which is as good or
// better there.  The first stage reads and the last one writes the plain
// layout the kernels load and store; the padded line fits in fft_ls(L).
template <int L>
__device__ __forceinline__ int fft_pad(int i) {
    return L >= 128 ? i + (i >> 4) : i + (i >> 3);
}

// tw: the stage twiddle table of load_twiddles (this stage's block at
// NS - plan_radix(L, 0), entry (t - 1) NS + k = w_L^(t k L / (NS RAD)))
template <typename R, bool INV, int RAD, int L, int NS, bool PIN, bool POUT>
__device__ __forceinline__ void stockham_stage_c(const Cx<R>* __restrict__ a, Cx<R>* __restrict__ b, int ls,
                                                 int nl, const Cx<R>* tw) {
    constexpr int nb = L / RAD;
    constexpr int tw_off = NS - plan_radix(L, 0);
    const int total = nb * nl;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int line = idx / nb;
        const int j = idx - line * nb;
        const int k = j % NS;
        const Cx<R>* src = a + line * ls;
        Cx<R>* dst = b + line * ls;
        Cx<R> v[RAD];
#pragma unroll
        for (int t = 0; t < RAD; ++t) v[t] = src[PIN ? fft_pad<L>(j + t * nb) : j + t * nb];
        if (NS > 1) {
#pragma unroll
            for (int t = 1; t < RAD; ++t) {
                Cx<R> w = tw[tw_off + (t - 1) * NS + k];
                if (INV) w.y = -w.y;
                v[t] = cmul(v[t], w);
            }
        }
        if (RAD == 2) dft2<Cx<R>, INV>(v[0], v[1]);
        else if (RAD == 3) dft3<R, INV>(v[0], v[1], v[2]);
        else if (RAD == 4) dft4<Cx<R>, INV>(v[0], v[1], v[2], v[3]);
        else dft8<R, INV>(v);
        const int out = (j - k) * RAD + k;
#pragma unroll
        for (int t = 0; t < RAD; ++t) dst[POUT ? fft_pad<L>(out + t * NS) : out + t * NS] = v[t];
    }
}

// ---------------------------------------------------------------------------
// Two-step FFT (FP32 lines of length L = P * Q).  With n = Q n1 + n2 and
// k = k1 + P k2,
//   X[k1 + P k2] = sum_n2 w_Q^(n2 k2) w_L^(n2 k1) sum_n1 w_P^(n1 k1) x[Q n1 + n2].
// Step 1, one work item per (line, n2): the P-point DFT over n1 in registers,
// the twiddle w_L^(n2 k1), each k1 stored in row k1 of a table with rows of
// Q + 1.  Step 2, one item per (line, k1): the Q-point DFT over n2 in
// registers, stored in natural order.  Every butterfly stays in registers:
// one shared-memory round trip and one barrier per step against one per
// radix stage of the Stockham passes, and about half their instructions
// (measured alone on this GPU: 1.8x the Stockham rate at L = 128, 2x at 256).
// Work items run line-fastest (LF) when a power-of-two count of 16 or more
// lines share the block: the lanes of a half-warp then hold 16 lines at the
// same offset, which the odd line stride puts on distinct banks.  The
// twiddles come as tw2[k1 * Q + n2] = w_L^(n2 k1) (load_twiddles lays the
// table out so for these lengths).
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R fmar(R a, R b, R c) {
    if constexpr (sizeof(R) == 4) return fmaf(a, b, c);
    else return fma(a, b, c);
}
template <typename R>
__device__ __forceinline__ Cx<R> cmulc(Cx<R> v, R wr, R wi) {  // v * (wr + i wi), constant factor
    return cx<R>(fmar<R>(v.x, wr, -(v.y * wi)), fmar<R>(v.x, wi, v.y * wr));
}

// 16-point DFT, natural order in and out: two 8-point DFTs of the even and
// odd elements, the odd ones times w16^k
template <typename R, bool INV>
__device__ __forceinline__ void dft16(Cx<R>* v) {
    Cx<R> e[8], o[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        e[i] = v[2 * i];
        o[i] = v[2 * i + 1];
    }
    dft8<R, INV>(e);
    dft8<R, INV>(o);
    const R c1 = (R)0.92387953251128675613, s1 = (R)0.38268343236508977173, h = (R)0.70710678118654752440;
    const R sg = INV ? (R)1 : (R)-1;  // w16^k = cos(2 pi k / 16) + i sg sin(2 pi k / 16)
    o[1] = cmulc<R>(o[1], c1, sg * s1);
    o[2] = cx<R>((o[2].x - sg * o[2].y) * h, (o[2].y + sg * o[2].x) * h);
    o[3] = cmulc<R>(o[3], s1, sg * c1);
    o[4] = INV ? cmul_pi(o[4]) : cmul_mi(o[4]);
    o[5] = cmulc<R>(o[5], -s1, sg * c1);
    o[6] = cx<R>((-o[6].x - sg * o[6].y) * h, (-o[6].y + sg * o[6].x) * h);
    o[7] = cmulc<R>(o[7], -c1, sg * s1);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = cadd(e[k], o[k]);
        v[k + 8] = csub(e[k], o[k]);
    }
}

// 12-point DFT, natural order: n = 4 n1 + n2, k = k1 + 3 k2; four 3-point
// DFTs, the twiddles w12^(n2 k1), three 4-point DFTs
template <typename R, bool INV>
__device__ __forceinline__ void dft12(Cx<R>* v) {
    Cx<R> y[4][3];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        Cx<R> a = v[n2], b = v[4 + n2], c = v[8 + n2];
        dft3<R, INV>(a, b, c);
        y[n2][0] = a;
        y[n2][1] = b;
        y[n2][2] = c;
    }
    const R r3 = (R)0.86602540378443864676, hf = (R)0.5;
    const R sg = INV ? (R)1 : (R)-1;
    y[1][1] = cmulc<R>(y[1][1], r3, sg * hf);             // w12^1
    y[1][2] = cmulc<R>(y[1][2], hf, sg * r3);             // w12^2
    y[2][1] = cmulc<R>(y[2][1], hf, sg * r3);             // w12^2
    y[2][2] = cmulc<R>(y[2][2], -hf, sg * r3);            // w12^4
    y[3][1] = INV ? cmul_pi(y[3][1]) : cmul_mi(y[3][1]);  // w12^3
    y[3][2] = cx<R>(-y[3][2].x, -y[3][2].y);              // w12^6
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
        Cx<R> a0 = y[0][k1], a1 = y[1][k1], a2 = y[2][k1], a3 = y[3][k1];
        dft4<Cx<R>, INV>(a0, a1, a2, a3);
        v[k1] = a0;
        v[k1 + 3] = a1;
        v[k1 + 6] = a2;
        v[k1 + 9] = a3;
    }
}

template <typename R, bool INV, int P>
__device__ __forceinline__ void dft_reg(Cx<R>* v) {
    if constexpr (P == 8) dft8<R, INV>(v);
    else if constexpr (P == 12) dft12<R, INV>(v);
    else if constexpr (P == 16) dft16<R, INV>(v);
    else static_assert(P == 8 || P == 12 || P == 16, "register DFT sizes 8, 12, 16");
}

// v * w (forward) or v * conj(w) (inverse), with fused multiply-adds
template <typename R, bool INV>
__device__ __forceinline__ Cx<R> twmul(Cx<R> v, Cx<R> w) {
    if (INV) return cx<R>(fmar<R>(v.x, w.x, v.y * w.y), fmar<R>(v.y, w.x, -(v.x * w.y)));
    return cx<R>(fmar<R>(v.x, w.x, -(v.y * w.y)), fmar<R>(v.x, w.y, v.y * w.x));
}

// Q of the factorisation L = P * Q of the two-step lengths (FP32); 0: the
// Stockham passes.  Measured in whole kicks on this GPU: the two-step passes
// are faster where the passes are bound by the SMs' issue rate (meshes of
// 96 to 128 cells per axis padded to 192 and 256, and batches), the Stockham
// passes where one wave of blocks makes them latency-bound (64-cell axes
// padded to 128: 0.228 against 0.221 ms per 2M / 64^3 kick).
__host__ __device__ constexpr int two_step_q(int L) {
    return L == 96 ? 12 : (L == 192 ? 16 : (L == 256 ? 16 : 0));
}

// ls >= fft_ls(L) >= P (Q + 1); a holds the input, b is scratch; the result
// is returned in a.  LF: nl is a power of two, lg its log2.  Called by every
// thread of the block; ends with a barrier.
template <typename R, bool INV, int L, bool LF>
__device__ __forceinline__ Cx<R>* fft_two_step(Cx<R>* a, Cx<R>* b, int ls, int nl, int lg, const Cx<R>* tw2) {
    constexpr int Q = two_step_q(L), P = L / Q;
    static_assert(Q > 0 && P * Q == L && P * (Q + 1) <= fft_ls(L), "two-step factorisation");
    for (int idx = threadIdx.x; idx < nl * Q; idx += blockDim.x) {
        int line, n2;
        if (LF) {
            n2 = idx >> lg;
            line = idx & (nl - 1);
        } else {
            line = idx / Q;
            n2 = idx - line * Q;
        }
        const Cx<R>* src = a + line * ls + n2;
        Cx<R> v[P];
#pragma unroll
        for (int n1 = 0; n1 < P; ++n1) v[n1] = src[n1 * Q];
        dft_reg<R, INV, P>(v);
        Cx<R>* dst = b + line * ls + n2;
        dst[0] = v[0];
#pragma unroll
        for (int k1 = 1; k1 < P; ++k1) dst[k1 * (Q + 1)] = twmul<R, INV>(v[k1], tw2[k1 * Q + n2]);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nl * P; idx += blockDim.x) {
        int line, k1;
        if (LF) {
            k1 = idx >> lg;
            line = idx & (nl - 1);
        } else {
            line = idx / P;
            k1 = idx - line * P;
        }
        const Cx<R>* src = b + line * ls + k1 * (Q + 1);
        Cx<R> u[Q];
#pragma unroll
        for (int n2 = 0; n2 < Q; ++n2) u[n2] = src[n2];
        dft_reg<R, INV, Q>(u);
        Cx<R>* dst = a + line * ls + k1;
#pragma unroll
        for (int k2 = 0; k2 < Q; ++k2) dst[k2 * P] = u[k2];
    }
    __syncthreads();
    return a;
}

template <typename R, bool INV, int L>
__device__ __forceinline__ Cx<R>* fft_two_step_any(Cx<R>* a, Cx<R>* b, int ls, int nl, const Cx<R>* tw2) {
    if (nl >= 16 && (nl & (nl - 1)) == 0) return fft_two_step<R, INV, L, true>(a, b, ls, nl, 31 - __clz(nl), tw2);
    return fft_two_step<R, INV, L, false>(a, b, ls, nl, 0, tw2);
}

// ls must be at least fft_ls(L)
template <typename R, bool INV, int L, int S, int NS>
__device__ __forceinline__ Cx<R>* fft_stages_c(Cx<R>* a, Cx<R>* b, int ls, int nl, const Cx<R>* tw) {
    constexpr int RAD = plan_radix(L, S);
    if constexpr (RAD == 0) {
        return a;
    } else {
        stockham_stage_c<R, INV, RAD, L, NS, (S > 0), (plan_radix(L, S + 1) != 0)>(a, b, ls, nl, tw);
        __syncthreads();
        return fft_stages_c<R, INV, L, S + 1, NS * RAD>(b, a, ls, nl, tw);
    }
}

// FFT of nl lines of length rp.L; a holds the input, b is scratch of the
// same shape.  Returns the buffer that holds the result.  Must be called by
// every thread of the block; ends with a barrier.
template <typename R, bool INV>
__device__ Cx<R>* fft_lines(Cx<R>* a, Cx<R>* b, int ls, int nl, const RadixPlan& rp, const Cx<R>* tw) {
    if constexpr (sizeof(R) == 4) {  // FP32: two register steps (tw laid out by load_twiddles)
        switch (rp.L) {
            case 96: return fft_two_step_any<R, INV, 96>(a, b, ls, nl, tw);
            case 192: return fft_two_step_any<R, INV, 192>(a, b, ls, nl, tw);
            case 256: return fft_two_step_any<R, INV, 256>(a, b, ls, nl, tw);
            default: break;
        }
    }
    switch (rp.L) {  // the padded lengths of meshes up to 256 per axis
        case 8: return fft_stages_c<R, INV, 8, 0, 1>(a, b, ls, nl, tw);
        case 12: return fft_stages_c<R, INV, 12, 0, 1>(a, b, ls, nl, tw);
        case 16: return fft_stages_c<R, INV, 16, 0, 1>(a, b, ls, nl, tw);
        case 24: return fft_stages_c<R, INV, 24, 0, 1>(a, b, ls, nl, tw);
        case 48: return fft_stages_c<R, INV, 48, 0, 1>(a, b, ls, nl, tw);
        case 96: return fft_stages_c<R, INV, 96, 0, 1>(a, b, ls, nl, tw);
        case 192: return fft_stages_c<R, INV, 192, 0, 1>(a, b, ls, nl, tw);
        case 384: return fft_stages_c<R, INV, 384, 0, 1>(a, b, ls, nl, tw);
        case 32: return fft_stages_c<R, INV, 32, 0, 1>(a, b, ls, nl, tw);
        case 64: return fft_stages_c<R, INV, 64, 0, 1>(a, b, ls, nl, tw);
        case 128: return fft_stages_c<R, INV, 128, 0, 1>(a, b, ls, nl, tw);
        case 256: return fft_stages_c<R, INV, 256, 0, 1>(a, b, ls, nl, tw);
        case 512: return fft_stages_c<R, INV, 512, 0, 1>(a, b, ls, nl, tw);
        default: break;
    }
    int Ns = 1;
    for (int s = 0; s < rp.nst; ++s) {
        const int r = rp.r[s], off = Ns - rp.r[0];
        if (r == 8) stockham_stage<R, INV, 8>(a, b, rp.L, ls, nl, Ns, tw, off);
        else if (r == 4) stockham_stage<R, INV, 4>(a, b, rp.L, ls, nl, Ns, tw, off);
        else if (r == 3) stockham_stage<R, INV, 3>(a, b, rp.L, ls, nl, Ns, tw, off);
        else stockham_stage<R, INV, 2>(a, b, rp.L, ls, nl, Ns, tw, off);
        __syncthreads();
        Cx<R>* t = a;
        a = b;
        b = t;
        Ns *= r;
    }
    return a;
}

// the radix of the next Stockham stage of a line with rem points left to
// split (the order of plan_radix / make_radix_plan: a 3 first, then 8s, a 4,
// a 2)
__host__ __device__ inline int next_radix(int rem) {
    return rem % 3 == 0 ? 3 : (rem % 8 == 0 ? 8 : (rem % 4 == 0 ? 4 : 2));
}

// The Stockham stage twiddle table: one block per stage after the first, in
// stage order -- the stage of NS points per butterfly group and radix RAD
// holds w_L^(t k L / (NS RAD)) at (t - 1) NS + k for t = 1 .. RAD - 1, k < NS,
// and starts at NS - R0 (R0 the first radix; L - R0 entries in all) -- so that
// lanes with consecutive k read consecutive entries (read from a table of
// w_L^m by m = t k L / (NS RAD), the 512-point stages put up to 8 lanes on one
// bank).  stage_tw_exponent gives the m of entry i < L - R0; the workspace's
// twiddle tables are laid out this way once, when it is initialised.
__host__ __device__ inline int stage_tw_exponent(int L, int i) {
    const int r0 = next_radix(L);
    const int g = i + r0;   // the stage of entry i: NS <= g < NS * RAD
    int ns = r0, rem = L / r0, r = next_radix(rem);
    while (ns * r <= g) {
        ns *= r;
        rem /= r;
        r = next_radix(rem);
    }
    const int rel = g - ns, t = rel / ns + 1, k = rel - (t - 1) * ns;
    return t * k * (L / (ns * r));
}

// Whether a line length of this precision takes the two-step form (its
// twiddle table then stays w_L^m in the workspace, the stage table otherwise).
template <typename R>
__host__ __device__ constexpr bool uses_two_step(int L) {
    return sizeof(R) == 4 && two_step_q(L) != 0;
}

// The twiddle table of fft_lines in shared memory (room for L entries) from
// the workspace's table src: for the two-step lengths of FP32 src[m] = w_L^m
// and tw2[k1 * Q + n2] = w_L^(n2 k1) is formed here; for the Stockham lengths
// src already holds the stage table and is copied.
template <typename R>
__device__ __forceinline__ void load_twiddles(Cx<R>* dst, const Cx<R>* src, int L) {
    if constexpr (sizeof(R) == 4) {
        const int Q = two_step_q(L);
        if (Q) {
            for (int i = threadIdx.x; i < L; i += blockDim.x) {
                const int k1 = i / Q, n2 = i - k1 * Q;
                dst[i] = src[k1 * n2];
            }
            return;
        }
    }
    for (int i = threadIdx.x; i < L; i += blockDim.x) dst[i] = src[i];
}

// Quotient and remainder of i = start, start + step, start + 2 step, ... by d,
// carried from one to the next: two divisions per thread instead of one per
// element in the line-staging loops (d is a run-time line length).
struct DivWalk {
    int q, r, dq, dr, d;
    __device__ __forceinline__ DivWalk(int start, int step, int d_) : d(d_) {
        q = start / d;
        r = start - q * d;
        dq = step / d;
        dr = step - dq * d;
    }
    __device__ __forceinline__ void next() {
        q += dq;
        r += dr;
        if (r >= d) {
            r -= d;
            ++q;
        }
    }
};

// Columns of a strided pass: the block's TK columns (TK a power of two) are
// consecutive entries of a flattened column index, thread t takes column
// t mod TK and rows t / TK, t / TK + blockDim / TK, ...; no division per element.
struct ColMap {
    int kk, r0, rs;
    __device__ __forceinline__ explicit ColMap(int TK) {
        const int lg = 31 - __clz(TK);
        kk = threadIdx.x & (TK - 1);
        r0 = threadIdx.x >> lg;
        rs = blockDim.x >> lg;
    }
};

}  // namespace ocsc
