// Per-particle stages of the space-charge kick.
//
//   frame   MAD -> lab Cartesian (coord_transform.py:57-96) and the sum of the
//           momenta for the mean-velocity frame (sc.py:224-231)
//   extent  rotation into that frame, z scaled by gamma0, and the min/max and
//           charge-weighted sums of the mesh geometry (sc.py:233, 172-181)
//   keys    grid coordinates X = xyz/steps - X_off and the NGP cell key
//           floor(X)+1 (sc.py:182-192)
//   kick    trilinear gather of the staggered field grids (sc.py:201-204),
//           the lab-frame kick (sc.py:244-250) and the transform back to MAD
//           (coord_transform.py:16-54), written into rparticles
//
// Two forms.  FP64 performs the reference's floating-point operations in the
// reference's order (explicit _rn intrinsics, so nothing is contracted into
// FMAs except where numpy's BLAS itself uses FMAs: the 3x3 rotations).  FP32
// computes every per-particle quantity in FP32 and writes the kick as small
// increments, each derived in closed form so that it carries no cancellation,
// added to the FP64 coordinates:
//     dE   = (2 p.dp + |dp|^2) / (E + E')
//     dx'  = dpx/pref, dy' = dpy/pref, ddelta = dE/pref
//     dtau = tau (pz E' - pz' E) / (E pz'), the bracket in a cancellation-free form
//     dx   = tau (dpx E - px dE) / (E E') + (px'/E') dtau      (same for y)
// Reductions are deterministic: a fixed grid, shuffle trees within blocks,
// per-block partials in HBM and a one-block finalize in a fixed order.
#include "sc_common.cuh"

namespace ocsc {

constexpr int PT = 256;  // threads per block of the particle kernels
constexpr unsigned FULL = 0xffffffffu;

// order-preserving map of a double onto uint64 (for integer atomics on doubles)
__device__ __forceinline__ unsigned long long ord64(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double unord64(unsigned long long u) {
    return __longlong_as_double((long long)((u >> 63) ? (u & 0x7fffffffffffffffull) : ~u));
}


// ---------------------------------------------------------------------------
// deterministic block reductions
// ---------------------------------------------------------------------------
// The shared scratch is passed as a sized array so that a scratch smaller
// than NV*32 elements is a compile-time error.
template <int NV, int SZ>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (&sm)[SZ]) {
    static_assert(SZ >= NV * 32, "block_sum: shared scratch too small");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c)
        for (int o = 16; o; o >>= 1) v[c] += __shfl_down_sync(FULL, v[c], o);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) sm[c * 32 + warp] = v[c];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            v[c] = lane < nw ? sm[c * 32 + lane] : 0.0;
            for (int o = 16; o; o >>= 1) v[c] += __shfl_down_sync(FULL, v[c], o);
        }
    }
    __syncthreads();
}

// error-free sum of two floats: s + e == a + b exactly (Knuth's TwoSum);
// written with _rn intrinsics so that nothing is contracted or reassociated
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (hi, lo) += (h2, l2) in double-float arithmetic (~48 significant bits)
__device__ __forceinline__ void df_add(float& hi, float& lo, float h2, float l2) {
    float s, e;
    two_sum(hi, h2, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, l2));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// Deterministic block sum of double-float pairs (hi, lo), as accurate as an
// FP64 reduction while the shuffles and adds stay on the FP32 pipes (this
// GPU's FP64 pipe issues a warp instruction in ~18 cycles, so FP64 block
// reductions dominate short kernels).  Thread 0 receives the sums in hi/lo.
template <int NV, int SZ>
__device__ __forceinline__ void block_sum_df(float (&hi)[NV], float (&lo)[NV], float (&sm)[SZ]) {
    static_assert(SZ >= NV * 64, "block_sum_df: shared scratch too small");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c)
        for (int o = 16; o; o >>= 1)
            df_add(hi[c], lo[c], __shfl_down_sync(FULL, hi[c], o), __shfl_down_sync(FULL, lo[c], o));
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            sm[c * 32 + warp] = hi[c];
            sm[(NV + c) * 32 + warp] = lo[c];
        }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            hi[c] = lane < nw ? sm[c * 32 + lane] : 0.f;
            lo[c] = lane < nw ? sm[(NV + c) * 32 + lane] : 0.f;
            for (int o = 16; o; o >>= 1)
                df_add(hi[c], lo[c], __shfl_down_sync(FULL, hi[c], o), __shfl_down_sync(FULL, lo[c], o));
        }
    }
    __syncthreads();
}
// the same for plain FP32 values (each thread's lo starts at 0)
template <int NV, int SZ>
__device__ __forceinline__ void block_sum_f2(const float (&v)[NV], float (&hi)[NV], float (&lo)[NV],
                                             float (&sm)[SZ]) {
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        hi[c] = v[c];
        lo[c] = 0.f;
    }
    block_sum_df<NV>(hi, lo, sm);
}

// block minimum or maximum of order-preserving 64-bit keys (ord64 of
// doubles) on the integer pipes; thread 0 receives the result
template <int NV, bool MAX, int SZ>
__device__ __forceinline__ void block_minmax_u64(unsigned long long (&v)[NV], unsigned long long (&sm)[SZ]) {
    static_assert(SZ >= NV * 32, "block_minmax_u64: shared scratch too small");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c)
        for (int o = 16; o; o >>= 1) {
            const unsigned long long w = __shfl_down_sync(FULL, v[c], o);
            v[c] = MAX ? (w > v[c] ? w : v[c]) : (w < v[c] ? w : v[c]);
        }
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) sm[c * 32 + warp] = v[c];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            v[c] = lane < nw ? sm[c * 32 + lane] : (MAX ? 0ull : ~0ull);
            for (int o = 16; o; o >>= 1) {
                const unsigned long long w = __shfl_down_sync(FULL, v[c], o);
                v[c] = MAX ? (w > v[c] ? w : v[c]) : (w < v[c] ? w : v[c]);
            }
        }
    }
    __syncthreads();
}

template <int NV, bool MAX, int SZ>
__device__ __forceinline__ void block_minmax(double (&v)[NV], double (&sm)[SZ]) {
    static_assert(SZ >= NV * 32, "block_minmax: shared scratch too small");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c)
        for (int o = 16; o; o >>= 1) {
            const double w = __shfl_down_sync(FULL, v[c], o);
            v[c] = MAX ? fmax(v[c], w) : fmin(v[c], w);
        }
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) sm[c * 32 + warp] = v[c];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            v[c] = lane < nw ? sm[c * 32 + lane] : (MAX ? -INFINITY : INFINITY);
            for (int o = 16; o; o >>= 1) {
                const double w = __shfl_down_sync(FULL, v[c], o);
                v[c] = MAX ? fmax(v[c], w) : fmin(v[c], w);
            }
        }
    }
    __syncthreads();
}

template <int NV, bool MAX, int SZ>
__device__ __forceinline__ void block_minmax_f(float (&v)[NV], float (&sm)[SZ]) {
    static_assert(SZ >= NV * 32, "block_minmax_f: shared scratch too small");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NV; ++c)
        for (int o = 16; o; o >>= 1) {
            const float w = __shfl_xor_sync(FULL, v[c], o);
            v[c] = MAX ? fmaxf(v[c], w) : fminf(v[c], w);
        }
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < NV; ++c) sm[c * 32 + warp] = v[c];
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        float r = lane < nw ? sm[c * 32 + lane] : (MAX ? -INFINITY : INFINITY);
        for (int o = 16; o; o >>= 1) {
            const float w = __shfl_xor_sync(FULL, r, o);
            r = MAX ? fmaxf(r, w) : fminf(r, w);
        }
        v[c] = r;  // every thread holds the block result
    }
    __syncthreads();
}

constexpr int PART_EXT = 11;

// ---------------------------------------------------------------------------
// FP64 transforms in the reference's operation order
// ---------------------------------------------------------------------------
// a / b from rb = RN(1/b): q = RN(a rb), then RN(q + (a - q b) rb) with the
// residual exact in one FMA (Markstein's correction).  Markstein's theorem
// gives RN(a/b) when the first q is within one ulp of a/b; from RN(1/b) it is
// within 1.5 ulp in the worst case, so the result is correctly rounded in
// every case tested (hundreds of millions, divisor significands near 1 and 2
// included) but not proven for all (a, b).  Three FP64 instructions instead of
// a division, which this GPU issues on its narrow FP64 pipe as a dozen; where
// a floor() follows the quotient, div_checked proves each result.
__device__ __forceinline__ double div_rb(double a, double b, double rb) {
    const double q = __dmul_rn(a, rb);
    return __fma_rn(__fma_rn(-q, b, a), rb, q);
}

// RN(a / b) for certain: div_rb's quotient q, kept only when the exact
// residual r = a - q b (one FMA) proves it, |r| < |b| ulp(q) / 2 -- then a/b
// lies within half an ulp of q.  The bound is |b| scaled by a power of two,
// built on the bit patterns and compared as integers (both non-negative).  A
// q that is a power of two (the spacing below it is half its ulp), zero, or
// near the ends of the exponent range goes to the IEEE division, and so does
// any q the test does not prove.  Used where floor() follows the quotient
// (the NGP keys), since a one-ulp change there can move a particle to the next
// cell.
__device__ __forceinline__ double div_checked(double a, double b, double rb) {
    const double q = div_rb(a, b, rb);
    const double r = __fma_rn(-q, b, a);
    const long long qb = __double_as_longlong(q);
    const long long bb = __double_as_longlong(b) & 0x7fffffffffffffffll;
    const int eq = (int)((qb >> 52) & 0x7ff), eb = (int)(bb >> 52);
    const int et = eb + eq - 1076;  // biased exponent of |b| 2^(eq - 1023 - 53)
    const long long thr = (bb & 0xfffffffffffffll) | ((long long)et << 52);
    const bool ok = (qb & 0xfffffffffffffll) != 0 && eq > 0 && eq < 2047 && eb > 0 && eb < 2047 && et > 0 &&
                    et < 2047 && (__double_as_longlong(r) & 0x7fffffffffffffffll) < thr;
    return ok ? q : __ddiv_rn(a, b);
}

// xxstg_2_xp_mad (coord_transform.py:57-96)
__device__ __forceinline__ void mad_to_cart64(const double r[6], const KickParams& kp, double xp[6]) {
    const double gamma = __dmul_rn(__dadd_rn(__dmul_rn(kp.betaref, r[5]), 1.0), kp.gamref);
    const double beta = __dsqrt_rn(__dsub_rn(1.0, __drcp_rn(__dmul_rn(gamma, gamma))));
    const double g = div_rb(__dmul_rn(gamma, beta), kp.grbr, kp.r_grbr);
    const double pz2pref = __dsqrt_rn(__dsub_rn(__dsub_rn(__dmul_rn(g, g), __dmul_rn(r[1], r[1])), __dmul_rn(r[3], r[3])));
    const double rpz = __drcp_rn(pz2pref);
    double u0 = div_rb(r[1], pz2pref, rpz), u1 = div_rb(r[3], pz2pref, rpz);
    const double nrm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(u0, u0), __dmul_rn(u1, u1)), 1.0));
    const double u2 = __drcp_rn(nrm);  // 1.0 / nrm
    u0 = div_rb(u0, nrm, u2);
    u1 = div_rb(u1, nrm, u2);
    xp[0] = __dsub_rn(r[0], __dmul_rn(__dmul_rn(u0, beta), r[4]));
    xp[1] = __dsub_rn(r[2], __dmul_rn(__dmul_rn(u1, beta), r[4]));
    xp[2] = __dmul_rn(__dmul_rn(-u2, beta), r[4]);
    xp[3] = __dmul_rn(__dmul_rn(__dmul_rn(u0, gamma), beta), kp.m_e_eV);
    xp[4] = __dmul_rn(__dmul_rn(__dmul_rn(u1, gamma), beta), kp.m_e_eV);
    xp[5] = __dmul_rn(__dmul_rn(__dmul_rn(u2, gamma), beta), kp.m_e_eV);
}

// xp_2_xxstg_mad (coord_transform.py:16-54); pos = lab x,y,z, p = new momenta
__device__ __forceinline__ void cart_to_mad64(const double pos[3], const double p[3], const KickParams& kp,
                                              double r[6]) {
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(p[0], p[0]), __dmul_rn(p[1], p[1])), __dmul_rn(p[2], p[2]));
    const double gamma = __dsqrt_rn(__dadd_rn(1.0, div_rb(s, kp.m2, kp.r_m2)));
    const double beta = __dsqrt_rn(__dsub_rn(1.0, __drcp_rn(__dmul_rn(gamma, gamma))));
    const double p0 = __dsqrt_rn(s);
    const double rp0 = __drcp_rn(p0);
    const double u0 = div_rb(p[0], p0, rp0), u1 = div_rb(p[1], p0, rp0), u2 = div_rb(p[2], p0, rp0);
    const double cdt = __ddiv_rn(-pos[2], __dmul_rn(beta, u2));
    r[0] = __dadd_rn(pos[0], __dmul_rn(__dmul_rn(beta, u0), cdt));
    r[2] = __dadd_rn(pos[1], __dmul_rn(__dmul_rn(beta, u1), cdt));
    r[5] = div_rb(__dsub_rn(div_rb(gamma, kp.gamref, kp.r_gamref), 1.0), kp.betaref, kp.r_betaref);
    r[4] = cdt;
    r[1] = div_rb(p[0], kp.pref, kp.r_pref);
    r[3] = div_rb(p[1], kp.pref, kp.r_pref);
}

// numpy's [N,3]@[3,3] row product: fma(a2,b2, fma(a1,b1, a0*b0))
__device__ __forceinline__ double dot3_blas(double a0, double a1, double a2, double b0, double b1, double b2) {
    return __fma_rn(a2, b2, __fma_rn(a1, b1, __dmul_rn(a0, b0)));
}

// ---------------------------------------------------------------------------
// FP64 <-> FP32 conversions on the integer pipes.  On this GPU the hardware
// conversions issue on the FP64 pipe, which the FP32 form keeps free for its
// six FP64 accumulations per particle.
// ---------------------------------------------------------------------------
// round-half-up to the nearest float (|error| <= 2^-24 relative); magnitudes
// below 2^-126 flush to zero, above FLT_MAX become infinity, NaN stays NaN.
// d2f_exact handles every exponent; d2f_nr only FP32's normal range, in five
// instructions, and d2f uses it with d2f_exact out of line (d2f_edge) for the
// rest.  All three give the same bits wherever they apply.
__device__ __forceinline__ float d2f_exact(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
    unsigned f;
    if (e <= 896) f = sign;
    else if (e >= 1151) f = sign | 0x7f800000u | ((e == 2047 && ((hi & 0xfffffu) | lo)) ? 0x400000u : 0u);
    else f = (sign | ((unsigned)(e - 896) << 23) | mant) + ((lo >> 28) & 1u);
    return __uint_as_float(f);
}
__device__ __noinline__ float d2f_edge(double d) { return d2f_exact(d); }
// d2f for a biased FP64 exponent of 897..1150 (the FP32 normal range): one
// funnel shift lines up the low eight exponent bits and 23 mantissa bits;
// adding 2^30 rebiases the exponent (-896 = +128 mod 256) and the first
// dropped bit rounds, its carry running into the exponent as in d2f_edge.
// range: the running unsigned maximum of (2|hi| - 2*897*2^20), below
// 2*254*2^20 iff every value converted so far was in range.
__device__ __forceinline__ float d2f_nr(double d, unsigned& range) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned t = __funnelshift_l(lo, hi, 3) + 0x40000000u + ((lo >> 28) & 1u);
    range = umax(range, hi * 2u - (897u << 21));
    return __uint_as_float((t & 0x7fffffffu) | (hi & 0x80000000u));
}
__device__ __forceinline__ bool d2f_range_ok(unsigned range) { return range < (254u << 21); }
// d2f_exact without its branches, for the kick: FP32's normal range as
// d2f_nr; magnitudes below it give +-0 and above it +-infinity (NaN too --
// the kick never sees either: the frame and extent latch non-finite and
// out-of-range data first).  Same bits as d2f_exact for every finite double.
__device__ __forceinline__ float d2f_kick(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
    const unsigned t = (__funnelshift_l(lo, hi, 3) + 0x40000000u + ((lo >> 28) & 1u)) & 0x7fffffffu;
    const unsigned f = mag < (897u << 20) ? 0u : (mag >= (1151u << 20) ? 0x7f800000u : t);
    return __uint_as_float(f | sign);
}
__device__ __forceinline__ float d2f(double d) {
    unsigned range = 0u;
    const float f = d2f_nr(d, range);
    return d2f_range_ok(range) ? f : d2f_edge(d);
}
// exact widening (float subnormals, which the kick never produces, read as
// 0); f2d_exact, f2d_nr and f2d split the exponents as the d2f forms do
__device__ __forceinline__ double f2d_exact(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned hi, lo;
    if (e == 0) { hi = sign; lo = 0u; }
    else if (e == 255) { hi = sign | 0x7ff00000u | (m >> 3); lo = m << 29; }
    else { hi = sign | ((e + 896u) << 20) | (m >> 3); lo = m << 29; }
    return __hiloint2double((int)hi, (int)lo);
}
__device__ __noinline__ double f2d_edge(float f) { return f2d_exact(f); }
// f2d for FP32 exponents 1..254 (rebiased by 896); range as in d2f_nr, below
// 2*254*2^23 iff every value was in range
__device__ __forceinline__ double f2d_nr(float f, unsigned& range) {
    const unsigned u = __float_as_uint(f);
    range = umax(range, u * 2u - (1u << 24));
    return __hiloint2double((int)((((u & 0x7fffffffu) >> 3) + 0x38000000u) | (u & 0x80000000u)), (int)(u << 29));
}
__device__ __forceinline__ bool f2d_range_ok(unsigned range) { return range < (254u << 24); }
__device__ __forceinline__ double f2d(float f) {
    unsigned range = 0u;
    const double d = f2d_nr(f, range);
    return f2d_range_ok(range) ? d : f2d_edge(f);
}

// the hardware's approximate reciprocal and square root (relative error
// ~1e-7)
__device__ __forceinline__ float rcpf(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sqrtf_fast(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Momenta (eV/c) and energy (eV) of one particle in FP32
// (coord_transform.py:64-72): gamma from delta, |p|^2 = (gamma^2 - 1) m^2,
// pz from |p|^2 - px^2 - py^2, with the approximate square root.  Where the
// FP32 form needs more than ~1e-7 relative accuracy it does not use these
// values directly: the mesh step and offset cancel a common scale of the
// positions (gamma0 scales both), the charge-weighted mean is taken of lab
// positions in which the momenta only enter a small correction (lab32), and
// NGP keys near a cell face are recomputed from FP64 coordinates (xyz_fine).
__device__ __forceinline__ void mom32(float xq, float yq, float d, const KickParams& kp, float& px, float& py,
                                      float& pz, float& E) {
    const float gamma = kp.gamref_f * fmaf(kp.betaref_f, d, 1.0f);
    const float g2 = fmaf(gamma, gamma, -1.0f) * kp.igrbr2_f;
    const float pz2 = sqrtf_fast(g2 - fmaf(xq, xq, yq * yq));
    px = xq * kp.pref_f;
    py = yq * kp.pref_f;
    pz = pz2 * kp.pref_f;
    E = gamma * kp.m_f;
}

// Lab position of one particle in FP32 (coord_transform.py:89-95): each
// coordinate is its MAD value plus a small correction, x - (px/E) tau and
// z = -tau + tau (1 - pz/E) with 1 - pz/E = (m^2 + pT^2) / ((E + pz) E),
// free of cancellation; the approximate reciprocal only touches the
// corrections.
__device__ __forceinline__ void lab32(float x, float y, float tau, float px, float py, float pz, float E,
                                      const KickParams& kp, float (&l)[3]) {
    const float iE = rcpf(E);
    const float s = tau * iE;
    l[0] = fmaf(-px, s, x);
    l[1] = fmaf(-py, s, y);
    const float k = (kp.m2_f + fmaf(px, px, py * py)) * rcpf((E + pz) * E);
    l[2] = fmaf(tau, k, -tau);
}
// rotated position in the beam frame, z scaled by gamma0 (sc.py:233)
__device__ __forceinline__ void rot32(const float (&l)[3], const float (&T)[3][3], float g0, float (&v)[3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) v[j] = fmaf(l[0], T[0][j], fmaf(l[1], T[1][j], l[2] * T[2][j]));
    v[2] *= g0;
}
// grid coordinate X = v/steps - X_off (sc.py:182-183) in FP32
__device__ __forceinline__ float grid32(float v, float istep, float off) { return fmaf(v, istep, -off); }

// 32-byte and 16-byte row accesses of G consecutive particles; a partial
// group (full == false) takes one element
template <int G>
__device__ __forceinline__ void ld_rows(const double* __restrict__ row, int64_t i, bool full, double (&a)[G]) {
    if constexpr (G == 4) {
        if (full) {
            asm("ld.global.nc.L1::no_allocate.v4.f64 {%0,%1,%2,%3}, [%4];"
                : "=d"(a[0]), "=d"(a[1]), "=d"(a[2]), "=d"(a[3])
                : "l"(row + i));
            return;
        }
    } else if constexpr (G == 2) {
        if (full) {
            const double2 v = __ldg(reinterpret_cast<const double2*>(row + i));
            a[0] = v.x;
            a[1] = v.y;
            return;
        }
    }
    a[0] = row[i];
#pragma unroll
    for (int w = 1; w < G; ++w) a[w] = 0.0;
}
template <int G>
__device__ __forceinline__ void st_rows(double* __restrict__ row, int64_t i, bool full, const double (&a)[G]) {
    if constexpr (G == 4) {
        if (full) {
            asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(row + i), "d"(a[0]), "d"(a[1]), "d"(a[2]),
                         "d"(a[3])
                         : "memory");
            return;
        }
    } else if constexpr (G == 2) {
        if (full) {
            *reinterpret_cast<double2*>(row + i) = make_double2(a[0], a[1]);
            return;
        }
    }
    row[i] = a[0];
}

// Group-wise particle loop: each thread takes G consecutive particles (one
// row access each), the last n mod G particles one per thread.  The loop
// strides over the blocks of the beam (vb), not of the launch.
#define GROUP_LOOP_BEGIN(n, G)                                                                    \
    const int64_t ngrp_ = (n) / (G);                                                              \
    const int64_t ntot_ = ngrp_ + ((n) - ngrp_ * (G));                                            \
    for (int64_t p_ = vb.x * (int64_t)blockDim.x + threadIdx.x; p_ < ntot_;                       \
         p_ += (int64_t)vb.nx * blockDim.x) {                                                     \
        const bool full_ = p_ < ngrp_;                                                            \
        const int64_t i0_ = full_ ? p_ * (G) : ngrp_ * (G) + (p_ - ngrp_);                        \
        const int W_ = full_ ? (G) : 1;
#define GROUP_LOOP_END }

// ---------------------------------------------------------------------------
// Bulk-copy (TMA) streaming of particle rows through shared memory, for the
// frame, extent and keys kernels.  A block walks its tiles of PT_TILE
// particles (local tile t is global tile vb.x + t * vb.nx); STAGES tile
// buffers rotate so that the loads of the next tiles are in flight while the
// block works on one.  Thread t takes particles 2t and 2t+1 of a tile.  A
// tile's copies cover a prefix whose byte length is a multiple of 16; the
// few particles after it (the end of the beam) are read directly.
// ---------------------------------------------------------------------------
constexpr int PT_TILE = 2 * PT;
constexpr int FR_STAGES = 4;  // tile buffers of the frame kernel (12 KB each)
constexpr int EX_STAGES = 2;  // tile buffers of the extent kernel (28 KB each)

struct BlockTiles {
    int64_t n, first, stride, mine;
    __device__ BlockTiles(int64_t n_, VBlk vb) : n(n_), first(vb.x), stride(vb.nx) {
        const int64_t nt = (n + PT_TILE - 1) / PT_TILE;
        mine = first < nt ? (nt - 1 - first) / stride + 1 : 0;
    }
    __device__ int64_t start(int64_t t) const { return (first + t * stride) * PT_TILE; }
    __device__ int count(int64_t t) const {
        const int64_t c = n - start(t);
        return (int)(c < PT_TILE ? c : PT_TILE);
    }
};

// Runs body(t, stage) for each of the block's tiles once its rows have
// landed in tile buffer `stage`; issue(t, stage, bar) (thread 0) starts the
// loads of local tile t.  Every thread of the block must call it; body must
// not synchronise the block.  Returns false if a wait gave up after `limit`
// tries, after waiting (with the full limit) for the loads still in flight.
template <int STAGES, typename Issue, typename Body>
__device__ __forceinline__ bool stream_tiles(const BlockTiles& T, uint64_t* bar, unsigned limit, Issue&& issue,
                                             Body&& body) {
    const bool lead = threadIdx.x == 0;
    if (lead) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bar[s], 1);
        mbar_init_fence();
    }
    __syncthreads();
    int64_t issued = T.mine < STAGES ? T.mine : STAGES;
    if (lead)
        for (int64_t t = 0; t < issued; ++t) issue(t, (int)t, &bar[t]);
    int64_t t = 0;
    bool failed = false;
    for (; t < T.mine; ++t) {
        const int s = (int)(t % STAGES);
        const bool ok = mbar_wait(&bar[s], (unsigned)((t / STAGES) & 1), limit);
        if (ok) body(t, s);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        // every thread is done with buffer s: it takes local tile t + STAGES
        if (lead && issued < T.mine) {
            issue(issued, s, &bar[s]);
            ++issued;
        }
    }
    if (failed && lead)
        for (int64_t u = t; u < issued; ++u) mbar_wait(&bar[u % STAGES], (unsigned)((u / STAGES) & 1));
    return !failed;
}

// shared memory of the streamed kernels: the tile buffers, then the barriers
constexpr size_t FR_SMEM = (size_t)FR_STAGES * 3 * PT_TILE * sizeof(double) + FR_STAGES * sizeof(uint64_t);
constexpr size_t EX_SMEM = (size_t)EX_STAGES * 7 * PT_TILE * sizeof(double) + EX_STAGES * sizeof(uint64_t);
static_assert(3 * (EX_SMEM + 1024 + 5 * 1024) <= 228 * 1024, "three extent blocks must fit an SM");

// ---------------------------------------------------------------------------
// last-block reductions: every block writes its partials, the last block to
// finish reduces all of them in block order (deterministic) and resets the
// counter for the next launch
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool arrive_last(unsigned int* counter, int nblk) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == (unsigned)nblk - 1u;
    }
    __syncthreads();
    return last;
}

// mean momentum -> basis T, gamma0, beta0 (sc.py:224-239, 243-248); called by
// the last block of a frame kernel with all per-block momentum sums in part
// Mean-velocity frame from the momentum sums (valid in thread 0); called by
// every thread of the last block.  The FP64 operations are the serial
// ones of sc.py:224-239, 243-248, spread over lanes: lane k of warp 0 takes
// component k of each basis vector and warp 1 the gamma0 chain, so the
// dependent FP64 divisions and square roots (very slow on this GPU's FP64
// pipe) form three short chains instead of one long one.  Each value goes
// through exactly the serial sequence of operations.
__device__ void frame_finish(const double (&acc)[3], const KickParams& kp, ScState* st) {
    __shared__ double s_acc[3];
    __shared__ double s_gamma0;
    __shared__ int s_bad1;
    if (threadIdx.x == 0) {
        st->done_frame = 0;
        st->kick_next = 0;  // the tile counter of this kick's gather + kick
        // the previous kick's outcome, kept before this kick resets the status
        if (st->status != SC_OK && st->first_error == SC_OK) st->first_error = st->status;
        for (int k = 0; k < 3; ++k) s_acc[k] = acc[k];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, k = lane < 3 ? lane : 0;
    if (warp > 1) return;
    const double nn = (double)kp.n;
    double t3k = __ddiv_rn(s_acc[k], nn);
    double t3[3] = {__shfl_sync(FULL, t3k, 0), __shfl_sync(FULL, t3k, 1), __shfl_sync(FULL, t3k, 2)};
    const double Pav = __dsqrt_rn(__fma_rn(t3[2], t3[2], __fma_rn(t3[1], t3[1], __dmul_rn(t3[0], t3[0]))));
    if (warp == 1) {
        if (lane == 0) {
            const double pm = __ddiv_rn(Pav, kp.m_e_eV);
            const double gamma0 = __dsqrt_rn(__dadd_rn(__dmul_rn(pm, pm), 1.0));
            const double beta0 = __dsqrt_rn(__dsub_rn(1.0, __drcp_rn(__dmul_rn(gamma0, gamma0))));
            st->Pav = Pav;
            st->gamma0 = gamma0;
            st->beta0 = beta0;
            st->kxy = __dmul_rn(kp.cdT, __dsub_rn(1.0, __dmul_rn(beta0, beta0)));
            st->kz = kp.cdT;
            st->g0f = (float)gamma0;
            st->ig0f = (float)(1.0 / gamma0);
            st->kxyf = (float)st->kxy;
            st->kzf = (float)kp.cdT;
            s_gamma0 = gamma0;
            s_bad1 = !(Pav > 0.0) || !isfinite(Pav) || !isfinite(gamma0);
        }
        asm volatile("bar.sync 1, 64;" ::: "memory");
        return;
    }
    t3k = __ddiv_rn(t3k, Pav);
    for (int j = 0; j < 3; ++j) t3[j] = __shfl_sync(FULL, t3k, j);
    // t1 = cross(ey, t3) = (t3z, 0, -t3x), normalised
    const double t1r[3] = {t3[2], 0.0, -t3[0]};
    const double n1 = __dsqrt_rn(__fma_rn(t1r[2], t1r[2], __fma_rn(t1r[1], t1r[1], __dmul_rn(t1r[0], t1r[0]))));
    const double t1k = __ddiv_rn(t1r[k], n1);
    const double t1[3] = {__shfl_sync(FULL, t1k, 0), __shfl_sync(FULL, t1k, 1), __shfl_sync(FULL, t1k, 2)};
    // t2 = cross(t3, t1)
    const double t2[3] = {__dsub_rn(__dmul_rn(t3[1], t1[2]), __dmul_rn(t3[2], t1[1])),
                          __dsub_rn(__dmul_rn(t3[2], t1[0]), __dmul_rn(t3[0], t1[2])),
                          __dsub_rn(__dmul_rn(t3[0], t1[1]), __dmul_rn(t3[1], t1[0]))};
    if (lane < 3) {
        st->T[lane][0] = t1[lane];
        st->T[lane][1] = t2[lane];
        st->T[lane][2] = t3[lane];
        st->Tf[lane][0] = (float)t1[lane];
        st->Tf[lane][1] = (float)t2[lane];
        st->Tf[lane][2] = (float)t3[lane];
    }
    asm volatile("bar.sync 1, 64;" ::: "memory");
    if (lane == 0) {
        int status = SC_OK;
        if (s_bad1 || !isfinite(s_gamma0) || !isfinite(t1[0]) || !isfinite(t2[1])) status = SC_ERR_NONFINITE;
        if (st->frame_timeout) {
            status = SC_ERR_TIMEOUT;
            st->frame_timeout = 0;
        }
        st->status = status;
    }
}

__device__ void frame_finalize(const double* part, int nblk, const KickParams& kp, ScState* st) {
    __shared__ double sm[3 * 32];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        for (int k = 0; k < 3; ++k) acc[k] += __ldcg(part + b * 3 + k);
    block_sum<3>(acc, sm);
    frame_finish(acc, kp, st);
}


// FP32 form: per-block momentum sums as double-float pairs (hi[3], lo[3]),
// reduced on the FP32 pipes
struct FramePart32 {
    float hi[3], lo[3];
};
__device__ void frame_finalize32(const FramePart32* part, int nblk, const KickParams& kp, ScState* st) {
    __shared__ float sm[3 * 64];
    float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        for (int k = 0; k < 3; ++k) df_add(hi[k], lo[k], __ldcg(&part[b].hi[k]), __ldcg(&part[b].lo[k]));
    block_sum_df<3>(hi, lo, sm);
    const double acc[3] = {(double)hi[0] + (double)lo[0], (double)hi[1] + (double)lo[1],
                           (double)hi[2] + (double)lo[2]};
    frame_finish(acc, kp, st);
}

// steps, X_off, potential scale, Green cache check (sc.py:172-186, 167)
// part layout per block (PART_EXT doubles): min[3], max[3], sum q*x[3], sum q, sum |q|
// lab_sums: the sums q*x are of lab positions (the FP32 extent); they are
// rotated into the beam frame and scaled by gamma0 here (a linear map, so
// the same charge-weighted mean)
// Mesh step, offset and derived constants from the extremes and charge
// moments (valid in thread 0); called by every thread of the last block.
// Lane k of warp 0 takes axis k with the serial FP64 operations of
// sc.py:172-186, so the divisions of the three axes run side by side.
__device__ void mesh_finish(const double (&mn)[3], const double (&mx)[3], const double (&qs)[5], const KickParams& kp,
                            ScState* st, double gamma_override, bool lab_sums) {
    __shared__ double s_mn[3], s_mx[3], s_qs[5];
    if (threadIdx.x == 0) {
        st->done_extent = 0;
        if (gamma_override > 0.0) {
            st->gamma0 = gamma_override;
            st->g0f = (float)gamma_override;
            st->ig0f = (float)(1.0 / gamma_override);
            st->status = SC_OK;
        }
        for (int k = 0; k < 3; ++k) {
            s_mn[k] = mn[k];
            s_mx[k] = mx[k];
        }
        for (int k = 0; k < 5; ++k) s_qs[k] = qs[k];
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    if (st->status != SC_OK) return;
    const int lane = threadIdx.x, k = lane < 3 ? lane : 0;
    double q3[3] = {s_qs[0], s_qs[1], s_qs[2]};
    if (lab_sums) {
        double r[3];
        for (int j = 0; j < 3; ++j) r[j] = fma(q3[2], st->T[2][j], fma(q3[1], st->T[1][j], q3[0] * st->T[0][j]));
        r[2] *= st->gamma0;
        for (int j = 0; j < 3; ++j) q3[j] = r[j];
    }
    const double qsum = s_qs[3];
    const int nm[3] = {kp.nx, kp.ny, kp.nz};
    // Every lane takes axis a = lane % 3 of the step; then group g = lane / 3
    // (0..4; lanes 15..31 repeat group 3) divides by it: g = 0 X_min,
    // g = 1 the charge-weighted mean (then / sum q), g = 2 1/step, g = 3 the
    // near-box ratio 5 h_max / step; in the second division group 4 forms the
    // FP32 form's potential scale phi_norm / (4 pi eps0 hx hy hz).  One SIMD
    // division serves all groups, so the chain holds three dependent
    // divisions instead of seven; each value is the same operation sequence
    // as the serial form.
    const int a = lane % 3, g = lane < 15 ? lane / 3 : 3;
    double XX = __dsub_rn(s_mx[a], s_mn[a]);
    if (!isnan(kp.mesh_scale)) XX = __dmul_rn(XX, kp.mesh_scale);
    const double stepa = __ddiv_rn(XX, (double)(nm[a] - 3));
    const double steps[3] = {__shfl_sync(FULL, stepa, 0), __shfl_sync(FULL, stepa, 1), __shfl_sync(FULL, stepa, 2)};
    const double hm = fmax(steps[0], fmax(steps[1], steps[2]));
    const double num = g == 0 ? s_mn[a] : g == 1 ? q3[a] : g == 2 ? 1.0 : __dmul_rn(5.0, hm);
    const double r1 = __ddiv_rn(num, stepa);
    const double pden = __dmul_rn(__dmul_rn(__dmul_rn(kp.four_pi_eps0, steps[0]), steps[1]), steps[2]);
    const double n2 = g == 4 ? kp.phi_norm : r1, d2 = g == 4 ? pden : qsum;
    const double r2 = __ddiv_rn(n2, d2);  // used by groups 1 and 4
    const double stepk = steps[k];
    const double xmin = __shfl_sync(FULL, r1, k);
    const double xmid = __shfl_sync(FULL, r2, 3 + k);
    const double istepk = __shfl_sync(FULL, r1, 6 + k);
    const double v = __shfl_sync(FULL, r1, 9 + k);
    const double scale = __shfl_sync(FULL, r2, 12);
    double xoffk = __dadd_rn(floor(__dsub_rn(xmin, xmid)), xmid);
    if (!isnan(kp.mesh_shift)) xoffk = __dadd_rn(xoffk, kp.mesh_shift);
    const bool badk = !(stepk > 0.0) || !isfinite(stepk) || !isfinite(xoffk);
    const bool bad = __any_sync(FULL, badk) || !(qsum != 0.0) || !isfinite(qsum);
    if (bad) {
        if (lane == 0) st->status = SC_ERR_DEGENERATE;
        return;
    }
    // near box of the hybrid Green's function along axis k (igf_box_of)
    int bk = v >= (double)nm[k] ? nm[k] : (int)ceil(v) + 1;
    if (bk > nm[k]) bk = nm[k];
    if (lane < 3) {
        st->steps[k] = stepk;
        st->xoff[k] = xoffk;
        st->isteps[k] = istepk;
        st->stepsf[k] = (float)stepk;
        st->istepsf[k] = (float)istepk;
        st->xofff[k] = (float)xoffk;
        st->igf_box[k] = bk;
        if (k < 2) st->igf_tbox[k] = igf_tbox_of(steps, k, nm[k]);
        if (k == 2) st->igf_line = igf_line_of(steps);
    }
    if (lane == 1) st->phi_norm = kp.phi_norm;
    if (lane == 2) {
        // fixed-point unit of the exact deposit: sum |q| * 2^S < 2^62, so no
        // cell (nor the total) can overflow a signed 64-bit accumulator
        int e2;
        frexp(s_qs[4], &e2);
        const int S = 62 - e2;
        st->qfix_shift = S;
        st->qfix_scale = ldexp(1.0, S);
        st->qfix_inv = (float)ldexp(1.0, -S);
    }
    if (lane == 0) {
        st->phi_denom = pden;
        st->phi_scalef = (float)scale;
        const bool same = steps[0] == st->igf_h[0] && steps[1] == st->igf_h[1] && steps[2] == st->igf_h[2];
        st->igf_rebuild = same ? 0 : 1;
        for (int j = 0; j < 3; ++j) st->igf_h[j] = steps[j];
    }
}

__device__ void mesh_finalize(const double* part, int nblk, const KickParams& kp, ScState* st, double gamma_override,
                              bool lab_sums = false) {
    __shared__ double sm[5 * 32];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    double qs[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        const double* o = part + b * PART_EXT;
        for (int k = 0; k < 3; ++k) {
            mn[k] = fmin(mn[k], __ldcg(o + k));
            mx[k] = fmax(mx[k], __ldcg(o + 3 + k));
            qs[k] += __ldcg(o + 6 + k);
        }
        qs[3] += __ldcg(o + 9);
        qs[4] += __ldcg(o + 10);
    }
    block_minmax<3, false>(mn, sm);
    block_minmax<3, true>(mx, sm);
    block_sum<5>(qs, sm);
    mesh_finish(mn, mx, qs, kp, st, gamma_override, lab_sums);
}

// FP32 form: per-block extremes as ord64 keys (integer min/max) and the
// charge moments of the lab positions as double-float pairs
struct ExtPart32 {
    unsigned long long mn[3], mx[3];
    float hi[5], lo[5];
};
static_assert(sizeof(ExtPart32) <= PART_EXT * sizeof(double), "ExtPart32 must fit a block's partial slot");
__device__ void mesh_finalize32(const ExtPart32* part, int nblk, const KickParams& kp, ScState* st) {
    __shared__ unsigned long long smu[3 * 32];
    __shared__ float smf[5 * 64];
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
    float hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            const unsigned long long a = __ldcg(&part[b].mn[k]), c = __ldcg(&part[b].mx[k]);
            mn[k] = a < mn[k] ? a : mn[k];
            mx[k] = c > mx[k] ? c : mx[k];
        }
        for (int k = 0; k < 5; ++k) df_add(hi[k], lo[k], __ldcg(&part[b].hi[k]), __ldcg(&part[b].lo[k]));
    }
    block_minmax_u64<3, false>(mn, smu);
    block_minmax_u64<3, true>(mx, smu);
    block_sum_df<5>(hi, lo, smf);
    const double dmn[3] = {unord64(mn[0]), unord64(mn[1]), unord64(mn[2])};
    const double dmx[3] = {unord64(mx[0]), unord64(mx[1]), unord64(mx[2])};
    double qs[5];
    for (int k = 0; k < 5; ++k) qs[k] = (double)hi[k] + (double)lo[k];
    mesh_finish(dmn, dmx, qs, kp, st, -1.0, true);
}

// ---------------------------------------------------------------------------
// frame: sum of momenta (+ FP64: lab coordinates stored for later stages)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(PT) k_frame64(const double* __restrict__ rp, KickParams kp,
                                                double* __restrict__ xp, double* __restrict__ part, ScState* st) {
    pdl_wait();
    __shared__ double sm[3 * 32];
    double acc[3] = {0.0, 0.0, 0.0};
    const int64_t n = kp.n, ld = kp.ld;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double r[6], c[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k] = rp[k * ld + i];
        mad_to_cart64(r, kp, c);
#pragma unroll
        for (int k = 0; k < 6; ++k) xp[k * n + i] = c[k];
        acc[0] += c[3];
        acc[1] += c[4];
        acc[2] += c[5];
    }
    block_sum<3>(acc, sm);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) part[blockIdx.x * 3 + k] = acc[k];
    if (arrive_last(&st->done_frame, gridDim.x)) frame_finalize(part, gridDim.x, kp, st);
}

// Pair-wise particle loop of the FP32 kernels: with VEC each thread takes two
// adjacent particles and moves every row with one 16-byte access (rows
// 16-byte aligned, even row stride); an odd last particle is taken alone.
// The loop strides over the blocks of the beam (vb), not of the launch.
#define PAIR_LOOP_BEGIN(n)                                                                        \
    const int64_t npair_ = VEC ? (n) / 2 : (n);                                                   \
    const int64_t ntot_ = npair_ + ((VEC && ((n) & 1)) ? 1 : 0);                                  \
    for (int64_t p_ = vb.x * (int64_t)blockDim.x + threadIdx.x; p_ < ntot_;                       \
         p_ += (int64_t)vb.nx * blockDim.x) {                                                     \
        const bool pair_ = VEC && p_ < npair_;                                                    \
        const int64_t i0_ = pair_ ? 2 * p_ : (VEC ? (n) - 1 : p_);                                \
        const int W_ = pair_ ? 2 : 1;
#define PAIR_LOOP_END }

__device__ __forceinline__ void ld_row(const double* __restrict__ row, int64_t i, bool pair, double& a, double& b) {
    if (pair) {
        const double2 v = __ldg(reinterpret_cast<const double2*>(row + i));
        a = v.x;
        b = v.y;
    } else {
        a = row[i];
        b = 0.0;
    }
}
__device__ __forceinline__ void st_row(double* __restrict__ row, int64_t i, bool pair, double a, double b) {
    if (pair) *reinterpret_cast<double2*>(row + i) = make_double2(a, b);
    else row[i] = a;
}
__device__ __forceinline__ void ld_rowf(const float* __restrict__ row, int64_t i, bool pair, float& a, float& b) {
    if (pair) {
        const float2 v = *reinterpret_cast<const float2*>(row + i);
        a = v.x;
        b = v.y;
    } else {
        a = row[i];
        b = 0.f;
    }
}
__device__ __forceinline__ void st_rowf(float* __restrict__ row, int64_t i, bool pair, float a, float b) {
    if (pair) *reinterpret_cast<float2*>(row + i) = make_float2(a, b);
    else row[i] = a;
}

// qzero != nullptr (batched kicks): the beam's blocks also clear its
// fixed-point charge grid of nzero cells for the deposit of this kick
template <bool VEC>
__device__ __forceinline__ void frame32_body(const double* __restrict__ rp, const KickParams& kp,
                                             double* __restrict__ part, ScState* st,
                                             unsigned long long* __restrict__ qzero, int64_t nzero, VBlk vb) {
    __shared__ float smf[3 * 64];
    if (qzero)
        for (int64_t i = vb.x * (int64_t)blockDim.x + threadIdx.x; i < nzero; i += (int64_t)vb.nx * blockDim.x)
            qzero[i] = 0ull;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const int64_t n = kp.n, ld = kp.ld;
    PAIR_LOOP_BEGIN(n)
    double xq[2], yq[2], d[2];
    ld_row(rp + ld, i0_, pair_, xq[0], xq[1]);
    ld_row(rp + 3 * ld, i0_, pair_, yq[0], yq[1]);
    ld_row(rp + 5 * ld, i0_, pair_, d[0], d[1]);
    for (int w = 0; w < W_; ++w) {
        float px, py, pz, E;
        mom32(d2f(xq[w]), d2f(yq[w]), d2f(d[w]), kp, px, py, pz, E);
        a0 += px;
        a1 += py;
        a2 += pz;
    }
    PAIR_LOOP_END
    const float a[3] = {a0, a1, a2};
    float hi[3], lo[3];
    block_sum_f2<3>(a, hi, lo, smf);
    FramePart32* fp = reinterpret_cast<FramePart32*>(part);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) {
            fp[vb.x].hi[k] = hi[k];
            fp[vb.x].lo[k] = lo[k];
        }
    if (arrive_last(&st->done_frame, vb.nx)) frame_finalize32(fp, vb.nx, kp, st);
}

// qzero != nullptr: also zeroes the nzero cells of the fixed-point charge
// grid for this kick's deposit
template <bool VEC>
__global__ void __launch_bounds__(PT, 4) k_frame32(const double* __restrict__ rp, KickParams kp,
                                                   double* __restrict__ part, ScState* st,
                                                   unsigned long long* __restrict__ qzero, int64_t nzero) {
    pdl_wait();
    frame32_body<VEC>(rp, kp, part, st, qzero, nzero, hw_vblk());
}

// frame32_body with the rows x', y', delta streamed through shared memory
// (rows 16-byte aligned, even stride)
__device__ __forceinline__ void frame32_tma_body(const double* __restrict__ rp, const KickParams& kp,
                                                 double* __restrict__ part, ScState* st,
                                                 unsigned long long* __restrict__ qzero, int64_t nzero, VBlk vb) {
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ float smf[3 * 64];
    double* buf = reinterpret_cast<double*>(smraw);  // [FR_STAGES][3][PT_TILE]
    uint64_t* bar = reinterpret_cast<uint64_t*>(buf + FR_STAGES * 3 * PT_TILE);
    if (qzero)
        for (int64_t i = vb.x * (int64_t)blockDim.x + threadIdx.x; i < nzero; i += (int64_t)vb.nx * blockDim.x)
            qzero[i] = 0ull;
    const int64_t n = kp.n, ld = kp.ld;
    const BlockTiles T(n, vb);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    auto addf = [&](float xq, float yq, float d) {
        float px, py, pz, E;
        mom32(xq, yq, d, kp, px, py, pz, E);
        a0 += px;
        a1 += py;
        a2 += pz;
    };
    auto add = [&](double xq, double yq, double d) { addf(d2f(xq), d2f(yq), d2f(d)); };
    auto issue = [&](int64_t t, int s, uint64_t* b) {
        const int64_t i0 = T.start(t);
        const unsigned bytes = (unsigned)(T.count(t) & ~1) * 8u;
        mbar_arrive_expect_tx(b, 3u * bytes);
        if (bytes)
            for (int r = 0; r < 3; ++r) bulk_load(buf + (s * 3 + r) * PT_TILE, rp + (2 * r + 1) * ld + i0, bytes, b);
    };
    auto body = [&](int64_t t, int s) {
        const int cnt = T.count(t), staged = cnt & ~1, j = 2 * threadIdx.x;
        const double* B = buf + s * 3 * PT_TILE;
        if (j + 1 < staged) {
            const double2 x = *reinterpret_cast<const double2*>(B + j);
            const double2 y = *reinterpret_cast<const double2*>(B + PT_TILE + j);
            const double2 d = *reinterpret_cast<const double2*>(B + 2 * PT_TILE + j);
            unsigned rg = 0u;  // one range check for both particles (d2f_nr)
            const float f[6] = {d2f_nr(x.x, rg), d2f_nr(y.x, rg), d2f_nr(d.x, rg),
                                d2f_nr(x.y, rg), d2f_nr(y.y, rg), d2f_nr(d.y, rg)};
            if (d2f_range_ok(rg)) {
                addf(f[0], f[1], f[2]);
                addf(f[3], f[4], f[5]);
            } else {
                add(x.x, y.x, d.x);
                add(x.y, y.y, d.y);
            }
        } else if (j < cnt) {
            const int64_t i = T.start(t) + j;
            add(rp[ld + i], rp[3 * ld + i], rp[5 * ld + i]);
        }
    };
    if (!stream_tiles<FR_STAGES>(T, bar, kp.wait_limit[0], issue, body) && threadIdx.x == 0)
        atomicExch(&st->frame_timeout, 1);
    const float a[3] = {a0, a1, a2};
    float hi[3], lo[3];
    block_sum_f2<3>(a, hi, lo, smf);
    FramePart32* fp = reinterpret_cast<FramePart32*>(part);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) {
            fp[vb.x].hi[k] = hi[k];
            fp[vb.x].lo[k] = lo[k];
        }
    if (arrive_last(&st->done_frame, vb.nx)) frame_finalize32(fp, vb.nx, kp, st);
}

__global__ void __launch_bounds__(PT, 4) k_frame32_tma(const double* __restrict__ rp, KickParams kp,
                                                       double* __restrict__ part, ScState* st,
                                                       unsigned long long* __restrict__ qzero, int64_t nzero) {
    pdl_wait();
    frame32_tma_body(rp, kp, part, st, qzero, nzero, hw_vblk());
}

// ---------------------------------------------------------------------------
// extent: rotated positions (z scaled by gamma0), min/max, charge moments
// ---------------------------------------------------------------------------
__device__ __forceinline__ void extent_block_out(double (&mn)[3], double (&mx)[3], double (&qs)[5],
                                                 double (&sm)[5 * 32], double* part, int bx) {
    block_minmax<3, false>(mn, sm);
    block_minmax<3, true>(mx, sm);
    block_sum<5>(qs, sm);
    if (threadIdx.x == 0) {
        double* o = part + bx * PART_EXT;
        for (int k = 0; k < 3; ++k) {
            o[k] = mn[k];
            o[3 + k] = mx[k];
            o[6 + k] = qs[k];
        }
        o[9] = qs[3];
        o[10] = qs[4];
    }
}

__global__ void __launch_bounds__(PT) k_extent64(const double* __restrict__ xp, const double* __restrict__ q,
                                                 KickParams kp, double* __restrict__ X, double* __restrict__ part,
                                                 ScState* st) {
    pdl_wait();
    __shared__ double sm[5 * 32];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    double qs[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const int64_t n = kp.n;
    const bool ok = st->status == SC_OK;
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = st->T[i][j];
    const double g0 = st->gamma0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ok && i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a0 = xp[i], a1 = xp[n + i], a2 = xp[2 * n + i];
        double v[3];
        for (int j = 0; j < 3; ++j) v[j] = dot3_blas(a0, a1, a2, T[0][j], T[1][j], T[2][j]);
        v[2] = __dmul_rn(v[2], g0);
        const double qi = q[i];
        for (int j = 0; j < 3; ++j) {
            X[j * kp.nX + i] = v[j];
            mn[j] = fmin(mn[j], v[j]);
            mx[j] = fmax(mx[j], v[j]);
            qs[j] += qi * v[j];
        }
        qs[3] += qi;
        qs[4] += fabs(qi);
    }
    extent_block_out(mn, mx, qs, sm, part, blockIdx.x);
    if (arrive_last(&st->done_extent, gridDim.x)) mesh_finalize(part, gridDim.x, kp, st, -1.0);
}

// Rotated position (z scaled by gamma0) of particle i with the FP64 form's
// operations, for the few particles whose FP32 position is too close to a
// cell face or to the extent to decide.  (Forming only the lab position's
// corrections in FP32 is not enough: at a few MeV the correction of z is a
// sizeable fraction of a cell, and its FP32 rounding of ~1e-8 cells put a
// particle 1.4e-8 cells from a face in the neighbouring cell.)  The result
// equals the FP64 form's position up to the rounding of the frame (T, gamma0),
// so the keys agree except for a particle within ~1e-14 cells of a face.
__device__ __forceinline__ void xyz_fine(const double* __restrict__ rp, int64_t ld, int64_t i, const KickParams& kp,
                                         const double (&T)[3][3], double g0, double v[3]) {
    // the FP64 form's operations: xxstg_2_xp_mad, the BLAS-order rotation
    // and the gamma0 product (k_frame64, k_extent64)
    double r[6], xp[6];
    for (int k = 0; k < 6; ++k) r[k] = rp[k * ld + i];
    mad_to_cart64(r, kp, xp);
    for (int j = 0; j < 3; ++j) v[j] = dot3_blas(xp[0], xp[1], xp[2], T[0][j], T[1][j], T[2][j]);
    v[2] = __dmul_rn(v[2], g0);
}
// A cheaper estimate of the same position, to ~1e-8 of a cell at a few MeV
// (~1e-11 at 100 MeV): each lab coordinate is its FP64 MAD value plus a small
// correction computed in FP32 (x - (px/E) tau, and z = -tau + tau (1 - pz/E)
// with 1 - pz/E = (m^2 + pT^2) / ((E + pz) E), free of cancellation), rotated
// in FP64.  Only for the near-face particles of a keys block beyond the
// KEYS_FINE that its list takes, inside the particle loop, where the FP64
// transform's registers would slow every particle.
// err (optional): a bound on |v - xyz_fine| per axis -- 2^-18 of each FP32
// correction (a few roundings of ~2^-24 each, the approximate reciprocals'
// ~2^-22, and margin) carried through the rotation.
__device__ __forceinline__ void xyz_fine32(const double* __restrict__ rp, int64_t ld, int64_t i,
                                           const KickParams& kp, const double (&T)[3][3], double g0, double v[3],
                                           double* err = nullptr) {
    const double x = rp[i], y = rp[2 * ld + i], tau = rp[4 * ld + i];
    float px, py, pz, E;
    mom32(d2f(rp[ld + i]), d2f(rp[3 * ld + i]), d2f(rp[5 * ld + i]), kp, px, py, pz, E);
    const float tf = d2f(tau), iE = rcpf(E);
    const float c0 = px * iE * tf, c1 = py * iE * tf;
    const double l0 = x - f2d(c0);
    const double l1 = y - f2d(c1);
    const float k = (kp.m2_f + fmaf(px, px, py * py)) * rcpf((E + pz) * E);
    const float c2 = tf * k;
    const double l2 = -tau + f2d(c2);
    for (int j = 0; j < 3; ++j) v[j] = fma(l2, T[2][j], fma(l1, T[1][j], l0 * T[0][j]));
    v[2] *= g0;
    if (err) {
        const double e0 = fabs((double)c0), e1 = fabs((double)c1), e2 = fabs((double)c2);
        for (int j = 0; j < 3; ++j)
            err[j] = ldexp(fma(e2, fabs(T[2][j]), fma(e1, fabs(T[1][j]), e0 * fabs(T[0][j]))), -18) *
                     (j == 2 ? g0 : 1.0);
    }
}


// FP32 extent.  Pass 1 computes the rotated positions in FP32, stores them and
// reduces FP32 extremes and charge moments.  Pass 2 re-walks the block's
// particles and evaluates in FP64 (xyz_fine) every particle whose
// FP32 coordinate lies within a rounding margin of the block's FP32 extreme:
// the FP64 extreme of the block is among them, so the mesh step equals the
// FP64 form's.
template <bool VEC>
__device__ __forceinline__ void extent32_body(const double* __restrict__ rp, const double* __restrict__ q,
                                              const KickParams& kp, float* __restrict__ X, double* __restrict__ part,
                                              ScState* st, VBlk vb) {
    __shared__ float smq[5 * 64];
    __shared__ float smf[3 * 32];
    __shared__ float bmin[3], bmax[3];
    __shared__ unsigned long long emin[3], emax[3];
    float mnf[3] = {INFINITY, INFINITY, INFINITY}, mxf[3] = {-INFINITY, -INFINITY, -INFINITY};
    float qsf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int64_t n = kp.n, ld = kp.ld, nX = kp.nX;
    const bool ok = st->status == SC_OK;
    float T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = st->Tf[i][j];
    const float g0 = st->g0f;
    if (ok) {
        PAIR_LOOP_BEGIN(n)
        float r[6][2], qq[2];
        for (int k = 0; k < 6; ++k) {
            double a, b;
            ld_row(rp + k * ld, i0_, pair_, a, b);
            r[k][0] = d2f(a);
            r[k][1] = d2f(b);
        }
        {
            double a, b;
            ld_row(q, i0_, pair_, a, b);
            qq[0] = d2f(a);
            qq[1] = d2f(b);
        }
        float v[3][2];
        for (int w = 0; w < W_; ++w) {
            float px, py, pz, E;
            mom32(r[1][w], r[3][w], r[5][w], kp, px, py, pz, E);
            float lw[3], vw[3];
            lab32(r[0][w], r[2][w], r[4][w], px, py, pz, E, kp, lw);
            rot32(lw, T, g0, vw);
            for (int j = 0; j < 3; ++j) v[j][w] = vw[j];
            const float qi = qq[w];
            for (int j = 0; j < 3; ++j) {  // charge moments of the lab positions
                mnf[j] = fminf(mnf[j], v[j][w]);
                mxf[j] = fmaxf(mxf[j], v[j][w]);
                qsf[j] = fmaf(qi, lw[j], qsf[j]);
            }
            qsf[3] += qi;
            qsf[4] += fabsf(qi);
        }
        for (int j = 0; j < 3; ++j) st_rowf(X + j * nX, i0_, pair_, v[j][0], v[j][1]);
        PAIR_LOOP_END
    }
    // float extremes reduce exactly in float; the sums in double
    block_minmax_f<3, false>(mnf, smf);
    block_minmax_f<3, true>(mxf, smf);
    float qhi[5], qlo[5];
    block_sum_f2<5>(qsf, qhi, qlo, smq);
    if (threadIdx.x == 0)
        for (int j = 0; j < 3; ++j) {
            bmin[j] = mnf[j];
            bmax[j] = mxf[j];
            emin[j] = ord64(INFINITY);
            emax[j] = ord64(-INFINITY);
        }
    __syncthreads();
    float tol[3];
    for (int j = 0; j < 3; ++j)  // 2^-18 of the coordinate scale: 64x the FP32 rounding bound of v
        tol[j] = ldexpf(fmaxf(fabsf(bmin[j]), fabsf(bmax[j])) + (bmax[j] - bmin[j]), -18);
    if (ok) {
        double Td[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) Td[a][b] = st->T[a][b];
        const double g0d = st->gamma0;
        // the same particles as pass 1 (same pair mapping), so the block's FP32
        // extremes bound them
        PAIR_LOOP_BEGIN(n)
        for (int w = 0; w < W_; ++w) {
            const int64_t i = i0_ + w;
            bool cand = false;
            for (int j = 0; j < 3; ++j) {
                const float v = X[j * nX + i];
                cand |= (v <= bmin[j] + tol[j]) || (v >= bmax[j] - tol[j]);
            }
            if (cand) {
                double v[3];
                xyz_fine(rp, ld, i, kp, Td, g0d, v);
                for (int j = 0; j < 3; ++j) {
                    if (X[j * nX + i] <= bmin[j] + tol[j]) atomicMin(&emin[j], ord64(v[j]));
                    if (X[j * nX + i] >= bmax[j] - tol[j]) atomicMax(&emax[j], ord64(v[j]));
                }
            }
        }
        PAIR_LOOP_END
    }
    __syncthreads();
    ExtPart32* ep = reinterpret_cast<ExtPart32*>(part);
    if (threadIdx.x == 0 && SC_IDX_OK(st, 12, vb.x, kp.n > 0 ? vb.nx : 0)) {
        for (int k = 0; k < 3; ++k) {
            ep[vb.x].mn[k] = emin[k];
            ep[vb.x].mx[k] = emax[k];
        }
        for (int k = 0; k < 5; ++k) {
            ep[vb.x].hi[k] = qhi[k];
            ep[vb.x].lo[k] = qlo[k];
        }
    }
    if (arrive_last(&st->done_extent, vb.nx)) mesh_finalize32(ep, vb.nx, kp, st);
}

template <bool VEC>
__global__ void __launch_bounds__(PT, 4) k_extent32(const double* __restrict__ rp, const double* __restrict__ q,
                                                    KickParams kp, float* __restrict__ X, double* __restrict__ part,
                                                    ScState* st) {
    pdl_wait();
    extent32_body<VEC>(rp, q, kp, X, part, st, hw_vblk());
}

constexpr int EX_SCAN = 4;  // tiles whose coordinates a pass-2 thread loads before checking them

// extent32_body with the six rows and the charges streamed through shared
// memory (rows and q 16-byte aligned, even stride).  Pass 2 is walked only
// by the threads whose own FP32 extreme lies within the margin of the
// block's: a particle of any other thread is farther from the block's
// extreme than that thread's extreme, so the candidates are the same.  Each
// such thread loads the coordinates of EX_SCAN tiles before it checks them,
// one round trip per EX_SCAN tiles instead of one per tile.
__device__ __forceinline__ void extent32_tma_body(const double* __restrict__ rp, const double* __restrict__ q,
                                                  const KickParams& kp, float* __restrict__ X,
                                                  double* __restrict__ part, ScState* st, VBlk vb) {
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ float smq[5 * 64];
    __shared__ float smf[3 * 32];
    __shared__ float bmin[3], bmax[3];
    __shared__ unsigned long long emin[3], emax[3];
    double* buf = reinterpret_cast<double*>(smraw);  // [EX_STAGES][7][PT_TILE]
    uint64_t* bar = reinterpret_cast<uint64_t*>(buf + EX_STAGES * 7 * PT_TILE);
    float mnf[3] = {INFINITY, INFINITY, INFINITY}, mxf[3] = {-INFINITY, -INFINITY, -INFINITY};
    float qsf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int64_t n = kp.n, ld = kp.ld, nX = kp.nX;
    const bool ok = !__syncthreads_or(st->status != SC_OK);
    float T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = st->Tf[i][j];
    const float g0 = st->g0f;
    const BlockTiles Tl(ok ? n : 0, vb);
    // one particle: rotated position, extremes and charge moments; returns v
    // f: the six coordinates and the charge rounded to FP32
    auto one = [&](const float (&f)[7], float (&v)[3]) {
        float px, py, pz, E;
        mom32(f[1], f[3], f[5], kp, px, py, pz, E);
        float l[3];
        lab32(f[0], f[2], f[4], px, py, pz, E, kp, l);
        rot32(l, T, g0, v);
        const float qi = f[6];
        for (int j = 0; j < 3; ++j) {  // charge moments of the lab positions
            mnf[j] = fminf(mnf[j], v[j]);
            mxf[j] = fmaxf(mxf[j], v[j]);
            qsf[j] = fmaf(qi, l[j], qsf[j]);
        }
        qsf[3] += qi;
        qsf[4] += fabsf(qi);
    };
    auto issue = [&](int64_t t, int s, uint64_t* b) {
        const int64_t i0 = Tl.start(t);
        const unsigned bytes = (unsigned)(Tl.count(t) & ~1) * 8u;
        mbar_arrive_expect_tx(b, 7u * bytes);
        if (bytes) {
            for (int k = 0; k < 6; ++k) bulk_load(buf + (s * 7 + k) * PT_TILE, rp + k * ld + i0, bytes, b);
            bulk_load(buf + (s * 7 + 6) * PT_TILE, q + i0, bytes, b);
        }
    };
    auto body = [&](int64_t t, int s) {
        const int cnt = Tl.count(t), staged = cnt & ~1, j = 2 * threadIdx.x;
        const int64_t i0 = Tl.start(t);
        const double* B = buf + s * 7 * PT_TILE;
        if (j + 1 < staged) {
            double r0[6], r1[6];
            for (int k = 0; k < 6; ++k) {
                const double2 v = *reinterpret_cast<const double2*>(B + k * PT_TILE + j);
                r0[k] = v.x;
                r1[k] = v.y;
            }
            const double2 qq = *reinterpret_cast<const double2*>(B + 6 * PT_TILE + j);
            float f0[7], f1[7];
            unsigned rg = 0u;  // one range check for both particles (d2f_nr)
            for (int k = 0; k < 6; ++k) {
                f0[k] = d2f_nr(r0[k], rg);
                f1[k] = d2f_nr(r1[k], rg);
            }
            f0[6] = d2f_nr(qq.x, rg);
            f1[6] = d2f_nr(qq.y, rg);
            if (!d2f_range_ok(rg)) {
                for (int k = 0; k < 6; ++k) {
                    f0[k] = d2f_edge(r0[k]);
                    f1[k] = d2f_edge(r1[k]);
                }
                f0[6] = d2f_edge(qq.x);
                f1[6] = d2f_edge(qq.y);
            }
            float v0[3], v1[3];
            one(f0, v0);
            one(f1, v1);
            for (int k = 0; k < 3; ++k) *reinterpret_cast<float2*>(X + k * nX + i0 + j) = make_float2(v0[k], v1[k]);
        } else if (j < cnt) {
            const int64_t i = i0 + j;
            float f[7];
            for (int k = 0; k < 6; ++k) f[k] = d2f(rp[k * ld + i]);
            f[6] = d2f(q[i]);
            float v[3];
            one(f, v);
            for (int k = 0; k < 3; ++k) X[k * nX + i] = v[k];
        }
    };
    const bool streamed = stream_tiles<EX_STAGES>(Tl, bar, kp.wait_limit[1], issue, body);
    if (!streamed && threadIdx.x == 0) atomicCAS(&st->status, SC_OK, SC_ERR_TIMEOUT);
    const float my_mn[3] = {mnf[0], mnf[1], mnf[2]}, my_mx[3] = {mxf[0], mxf[1], mxf[2]};
    // float extremes reduce exactly in float; the sums in double
    block_minmax_f<3, false>(mnf, smf);
    block_minmax_f<3, true>(mxf, smf);
    float qhi[5], qlo[5];
    block_sum_f2<5>(qsf, qhi, qlo, smq);
    if (threadIdx.x == 0)
        for (int j = 0; j < 3; ++j) {
            bmin[j] = mnf[j];
            bmax[j] = mxf[j];
            emin[j] = ord64(INFINITY);
            emax[j] = ord64(-INFINITY);
        }
    __syncthreads();
    float tol[3];
    bool mine = false;
    for (int j = 0; j < 3; ++j) {  // 2^-18 of the coordinate scale: 64x the FP32 rounding bound of v
        tol[j] = ldexpf(fmaxf(fabsf(bmin[j]), fabsf(bmax[j])) + (bmax[j] - bmin[j]), -18);
        mine |= (my_mn[j] <= bmin[j] + tol[j]) || (my_mx[j] >= bmax[j] - tol[j]);
    }
    if (ok && streamed && mine) {
        double Td[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) Td[a][b] = st->T[a][b];
        const double g0d = st->gamma0;
        for (int64_t t0 = 0; t0 < Tl.mine; t0 += EX_SCAN) {
            float xv[EX_SCAN][2][3];
#pragma unroll
            for (int u = 0; u < EX_SCAN; ++u)
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    const int64_t t = t0 + u;
                    const int jj = 2 * threadIdx.x + w;
                    const bool valid = t < Tl.mine && jj < Tl.count(t);
                    const int64_t i = valid ? Tl.start(t) + jj : 0;
#pragma unroll
                    for (int j = 0; j < 3; ++j) xv[u][w][j] = valid ? X[j * nX + i] : NAN;
                }
            // the extremes each particle may be: 6 bits per particle (min x, y, z; max x, y, z)
            unsigned long long sides = 0;
#pragma unroll
            for (int u = 0; u < EX_SCAN; ++u)
#pragma unroll
                for (int w = 0; w < 2; ++w)
#pragma unroll
                    for (int j = 0; j < 3; ++j) {  // NaN (no particle) is no candidate
                        const int b = 6 * (2 * u + w);
                        if (xv[u][w][j] <= bmin[j] + tol[j]) sides |= 1ull << (b + j);
                        if (xv[u][w][j] >= bmax[j] - tol[j]) sides |= 8ull << (b + j);
                    }
            while (sides) {
                const int p = (__ffsll((long long)sides) - 1) / 6;  // first candidate: particle p of the chunk
                const unsigned sd = (unsigned)(sides >> (6 * p)) & 63u;
                sides &= ~(63ull << (6 * p));
                const int64_t i = Tl.start(t0 + p / 2) + 2 * threadIdx.x + (p & 1);
                double v[3];
                xyz_fine(rp, ld, i, kp, Td, g0d, v);
                for (int j = 0; j < 3; ++j) {
                    if (sd & (1u << j)) atomicMin(&emin[j], ord64(v[j]));
                    if (sd & (8u << j)) atomicMax(&emax[j], ord64(v[j]));
                }
            }
        }
    }
    __syncthreads();
    ExtPart32* ep = reinterpret_cast<ExtPart32*>(part);
    if (threadIdx.x == 0 && SC_IDX_OK(st, 12, vb.x, kp.n > 0 ? vb.nx : 0)) {
        for (int k = 0; k < 3; ++k) {
            ep[vb.x].mn[k] = emin[k];
            ep[vb.x].mx[k] = emax[k];
        }
        for (int k = 0; k < 5; ++k) {
            ep[vb.x].hi[k] = qhi[k];
            ep[vb.x].lo[k] = qlo[k];
        }
    }
    if (arrive_last(&st->done_extent, vb.nx)) mesh_finalize32(ep, vb.nx, kp, st);
}

__global__ void __launch_bounds__(PT, 3) k_extent32_tma(const double* __restrict__ rp, const double* __restrict__ q,
                                                        KickParams kp, float* __restrict__ X,
                                                        double* __restrict__ part, ScState* st) {
    pdl_wait();
    extent32_tma_body(rp, q, kp, X, part, st, hw_vblk());
}

// el_field entry: X given as [n][3] rotated positions; z scaled by gamma in place
template <typename R>
__global__ void __launch_bounds__(PT) k_extent_xyz(double* __restrict__ Xin, const double* __restrict__ q, KickParams kp,
                                                   double gamma, R* __restrict__ X, double* __restrict__ part,
                                                   ScState* st) {
    pdl_wait();
    __shared__ double sm[5 * 32];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    double qs[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const int64_t n = kp.n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v[3] = {Xin[3 * i], Xin[3 * i + 1], __dmul_rn(Xin[3 * i + 2], gamma)};
        Xin[3 * i + 2] = v[2];
        const double qi = q[i];
        for (int j = 0; j < 3; ++j) {
            X[j * kp.nX + i] = (R)v[j];
            mn[j] = fmin(mn[j], v[j]);
            mx[j] = fmax(mx[j], v[j]);
            qs[j] += qi * v[j];
        }
        qs[3] += qi;
        qs[4] += fabs(qi);
    }
    extent_block_out(mn, mx, qs, sm, part, blockIdx.x);
    if (arrive_last(&st->done_extent, gridDim.x)) mesh_finalize(part, gridDim.x, kp, st, gamma);
}

// potential entry: explicit spacing
__global__ void k_set_mesh(ScState* st, double hx, double hy, double hz, KickParams kp) {
    pdl_wait();
    st->status = SC_OK;
    st->steps[0] = hx;
    st->steps[1] = hy;
    st->steps[2] = hz;
    st->stepsf[0] = (float)hx;
    st->stepsf[1] = (float)hy;
    st->stepsf[2] = (float)hz;
    st->isteps[0] = __ddiv_rn(1.0, hx);
    st->isteps[1] = __ddiv_rn(1.0, hy);
    st->isteps[2] = __ddiv_rn(1.0, hz);
    st->phi_denom = __dmul_rn(__dmul_rn(__dmul_rn(kp.four_pi_eps0, hx), hy), hz);
    st->phi_scalef = (float)(kp.phi_norm / st->phi_denom);
    st->phi_norm = kp.phi_norm;
    const double h[3] = {hx, hy, hz};
    igf_box_of(h, kp.nx, kp.ny, kp.nz, st->igf_box);
    st->igf_line = igf_line_of(h);
    st->igf_tbox[0] = igf_tbox_of(h, 0, kp.nx);
    st->igf_tbox[1] = igf_tbox_of(h, 1, kp.ny);
    const bool same = hx == st->igf_h[0] && hy == st->igf_h[1] && hz == st->igf_h[2];
    st->igf_rebuild = same ? 0 : 1;
    st->igf_h[0] = hx;
    st->igf_h[1] = hy;
    st->igf_h[2] = hz;
}

// ---------------------------------------------------------------------------
// keys: X = xyz/steps - X_off, key = (Xi*ny + Yi)*nz + Zi with Xi = floor(X)+1
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool key_of(double fx, double fy, double fz, const KickParams& kp, uint32_t& key) {
    const bool in = fx >= 0 && fy >= 0 && fz >= 0 && fx < kp.nx && fy < kp.ny && fz < kp.nz;
    key = in ? ((uint32_t)fx * (uint32_t)kp.ny + (uint32_t)fy) * (uint32_t)kp.nz + (uint32_t)fz : 0u;
    return in;
}

// FP64: whether 0 <= c <= hi (c = -0.0 included, NaN excluded) and floor(c)
// for such c, both on the bit pattern: the order of non-negative doubles is
// the order of their bits, and the integer part is the significand shifted
// by the exponent.  Equal to the double compares and floor(), without the
// FP64 pipe, which this GPU issues at a fraction of its integer rate.
__device__ __forceinline__ bool in_range64(double c, double hi) {
    const long long b = __double_as_longlong(c);
    return (b >= 0 || b == (long long)0x8000000000000000ull) && b <= __double_as_longlong(hi);
}
__device__ __forceinline__ int floor_nonneg64(double c) {  // 0 <= c < 2^31
    const long long b = __double_as_longlong(c);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < 0) return 0;
    const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    return (int)(m >> (52 - e));
}

// c = floor(g) + 1 and whether 0 <= c < n (key_of's test), for a double grid
// coordinate g, on its bit pattern: +-0 gives 1; 0 < g < n - 1 gives
// floor(g) + 1; -1 <= g < 0 gives 0; anything else (NaN, infinities
// included) is out of the mesh.
__device__ __forceinline__ bool cell_of64(double g, int n, uint32_t& c) {
    const long long b = __double_as_longlong(g);
    if ((b << 1) == 0) {
        c = 1u;
        return n > 1;
    }
    if (b > 0) {
        if (b >= __double_as_longlong((double)(n - 1))) return false;
        c = (uint32_t)floor_nonneg64(g) + 1u;
        return true;
    }
    if ((b & 0x7FFFFFFFFFFFFFFFll) > 0x3FF0000000000000ll) return false;
    c = 0u;
    return true;
}

__global__ void __launch_bounds__(PT) k_keys64(double* __restrict__ X, uint32_t* __restrict__ keys, KickParams kp,
                                               ScState* st) {
    pdl_wait();
    if (st->status) return;
    const int64_t n = kp.n;
    const double s0 = st->steps[0], s1 = st->steps[1], s2 = st->steps[2];
    // isteps = RN(1/steps): the quotients below are the correctly rounded X / steps (div_checked)
    const double r0 = st->isteps[0], r1 = st->isteps[1], r2 = st->isteps[2];
    const double o0 = st->xoff[0], o1 = st->xoff[1], o2 = st->xoff[2];
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t nX = kp.nX;
        const double g0 = __dsub_rn(div_checked(X[i], s0, r0), o0);
        const double g1 = __dsub_rn(div_checked(X[nX + i], s1, r1), o1);
        const double g2 = __dsub_rn(div_checked(X[2 * nX + i], s2, r2), o2);
        uint32_t c0, c1, c2;
        const bool in = cell_of64(g0, kp.nx, c0) & cell_of64(g1, kp.ny, c1) & cell_of64(g2, kp.nz, c2);
        bad |= !in;
        keys[i] = in ? (c0 * (uint32_t)kp.ny + c1) * (uint32_t)kp.nz + c2 : 0u;
        X[i] = g0;
        X[nX + i] = g1;
        X[2 * nX + i] = g2;
    }
    if (bad) atomicCAS(&st->status, SC_OK, SC_ERR_NONFINITE);
}

__device__ __forceinline__ bool key_of_f(float fx, float fy, float fz, const KickParams& kp, uint32_t& key) {
    const bool in = fx >= 0.f && fy >= 0.f && fz >= 0.f && fx < (float)kp.nx && fy < (float)kp.ny && fz < (float)kp.nz;
    key = in ? ((uint32_t)fx * (uint32_t)kp.ny + (uint32_t)fy) * (uint32_t)kp.nz + (uint32_t)fz : 0u;
    return in;
}

// q * 2^S rounded to an integer, on the integer pipes (|q| 2^S < 2^62)
// One charge into the fixed-point grid: a reduction without a return value
// (red), so the thread does not wait for the L2 round trip of the atomic.
// (atomicAdd with its result unused compiles to an atom that returns it,
// and the next use of its register waits for the reply.)  Integer addition
// in any order gives the same grid.
__device__ __forceinline__ void deposit_fixed(unsigned long long* p, long long v) {
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(p), "l"((unsigned long long)v) : "memory");
}

__device__ __forceinline__ long long to_fixed(double q, int S) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) return 0;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int sh = e - 1075 + S;
    unsigned long long v;
    if (sh >= 0) v = sh > 10 ? 0x3fffffffffffffffull : (m << sh);
    else if (sh < -63) v = 0;
    else v = (m + (1ull << (-sh - 1))) >> (-sh);
    return (b >> 63) ? -(long long)v : (long long)v;
}

// NGP key of a near-face particle, equal to the FP64 form's: the grid
// coordinate from the cheap estimate when every axis is farther from a face
// than the estimate's error bound (plus 1e-12 cells for the FP64 roundings),
// else from the FP64 form's operations.  Returns false outside the mesh.
__device__ __forceinline__ bool key_fine(const double* __restrict__ rp, int64_t ld, int64_t i, const KickParams& kp,
                                         const ScState* st, uint32_t& key, float (&gf)[3]) {
    double T[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) T[a][b] = st->T[a][b];
    double xv[3], err[3], g[3];
    xyz_fine32(rp, ld, i, kp, T, st->gamma0, xv, err);
    bool sure = true;
    for (int j = 0; j < 3; ++j) {  // the FP64 form's grid coordinate (k_keys64)
        g[j] = __dsub_rn(div_checked(xv[j], st->steps[j], st->isteps[j]), st->xoff[j]);
        const double d = fabs(g[j] - rint(g[j]));
        sure &= d > fma(err[j], st->isteps[j], 1e-12);
    }
    if (!sure) {
        xyz_fine(rp, ld, i, kp, T, st->gamma0, xv);
        for (int j = 0; j < 3; ++j) g[j] = __dsub_rn(div_checked(xv[j], st->steps[j], st->isteps[j]), st->xoff[j]);
    }
    for (int j = 0; j < 3; ++j) gf[j] = (float)g[j];
    return key_of(floor(g[0]) + 1, floor(g[1]) + 1, floor(g[2]) + 1, kp, key);
}

constexpr int KEYS_FINE = 1024;

// FP32 grid coordinates with an explicit rounding margin; a particle whose
// coordinate lies within the margin of a cell face is recomputed with the
// FP64 form's operations (xyz_fine, then X / step - X_off as k_keys64), so
// its key equals the FP64 form's key unless it lies within the rounding of
// the frame (~1e-14 cells) of the face (key_fine: the cheap estimate
// xyz_fine32 decides unless it lies within its error bound of a face).  A
// block lists up to KEYS_FINE such particles (about 0.4% of a beam's
// particles are near a face; a block holds a few thousand); beyond that, in
// degenerate beams only, the rest take the cheap estimate alone.
// rp == nullptr (el_field entry) keeps the FP32 result.
// qfix != nullptr: the deposit -- each charge, in units of 2^-S, is added to
// its cell with a 64-bit integer atomic.  Integer addition is exact and
// associative, so the charge grid does not depend on the order of the
// atomics: deterministic, the same alone and in a batch.
template <bool VEC>
__device__ __forceinline__ void keys32_body(float* __restrict__ X, uint32_t* __restrict__ keys,
                                            const double* __restrict__ rp, const double* __restrict__ q,
                                            unsigned long long* __restrict__ qfix, const KickParams& kp, ScState* st,
                                            VBlk vb) {
    // particles within the margin of a cell face, evaluated in FP64 after the
    // loop, one per thread (KEYS_FINE of them per block; more go inline)
    __shared__ uint32_t s_fine[KEYS_FINE];
    __shared__ int s_nfine;
    if (threadIdx.x == 0) s_nfine = 0;
    if (__syncthreads_or(st->status != SC_OK)) return;  // the same decision in every thread of the block
    const int64_t n = kp.n, ld = kp.ld, nX = kp.nX;
    float of[3], is[3];
    for (int j = 0; j < 3; ++j) {
        of[j] = st->xofff[j];
        is[j] = st->istepsf[j];
    }
    const float ig0 = st->ig0f, g0 = st->g0f;
    const int S = st->qfix_shift;
    bool bad = false;
    // the pair loop of PAIR_LOOP_BEGIN, KG pairs per thread per round: the
    // loads of all KG pairs are issued before the first is processed, so a
    // thread keeps KG times the bytes in flight
    constexpr int KG = 2;
    const int64_t npair_ = VEC ? n / 2 : n;
    const int64_t ntot_ = npair_ + ((VEC && (n & 1)) ? 1 : 0);
    const int64_t pstride_ = (int64_t)vb.nx * blockDim.x;
    for (int64_t pg_ = vb.x * (int64_t)blockDim.x + threadIdx.x; pg_ < ntot_; pg_ += KG * pstride_) {
        unsigned slow = 0u;  // bit 2u + w: particle w of pair u takes the estimate after the round
        float vg[KG][3][2];
        double qg[KG][2];
#pragma unroll
        for (int u = 0; u < KG; ++u) {
            const int64_t p_ = pg_ + u * pstride_;
            const bool pair_ = VEC && p_ < npair_;
            const int64_t i0_ = pair_ ? 2 * p_ : (VEC ? n - 1 : p_);
            qg[u][0] = qg[u][1] = 0.0;
            if (p_ < ntot_) {
                for (int j = 0; j < 3; ++j) ld_rowf(X + j * nX, i0_, pair_, vg[u][j][0], vg[u][j][1]);
                if (qfix) ld_row(q, i0_, pair_, qg[u][0], qg[u][1]);
            }
        }
#pragma unroll
        for (int u = 0; u < KG; ++u) {
            const int64_t p_ = pg_ + u * pstride_;
            if (p_ >= ntot_) break;
            const bool pair_ = VEC && p_ < npair_;
            const int64_t i0_ = pair_ ? 2 * p_ : (VEC ? n - 1 : p_);
            const int W_ = pair_ ? 2 : 1;
            float (&v)[3][2] = vg[u];
            double (&qq)[2] = qg[u];
            uint32_t key2[2] = {0u, 0u};
            float g2[3][2];
            for (int w = 0; w < W_; ++w) {
                const int64_t i = i0_ + w;
                const float v0 = v[0][w], v1 = v[1][w], v2 = v[2][w];
                const float nrm = sqrtf_fast(fmaf(v0, v0, fmaf(v1, v1, (v2 * ig0) * (v2 * ig0))));  // |lab position|
                float g[3] = {grid32(v0, is[0], of[0]), grid32(v1, is[1], of[1]), grid32(v2, is[2], of[2])};
                bool amb = false;
                for (int j = 0; j < 3; ++j) {
                    const float scale = (j == 2 ? nrm * g0 : nrm) * is[j] + fabsf(of[j]) + 1.0f;
                    // 16 units in the last place of the scale: 2x the error bound of g
                    // (FP32 position with approximate momenta, product, difference)
                    const float tol = ldexpf(scale, -19);
                    const float f = g[j] - floorf(g[j]);
                    amb |= !(f >= tol && f <= 1.0f - tol);
                }
                uint32_t key = 0u;
                bool deferred = false;
                if (amb && rp) {
                    const int slot = atomicAdd(&s_nfine, 1);
                    if (slot < KEYS_FINE) s_fine[slot] = (uint32_t)i;  // n < 2^31
                    else slow |= 1u << (2 * u + w);                    // the list is full: after this round
                    deferred = true;
                }
                if (!deferred) {
                    bad |= !key_of_f(floorf(g[0]) + 1.f, floorf(g[1]) + 1.f, floorf(g[2]) + 1.f, kp, key);
                    if (qfix && SC_IDX_OK(st, 11, key, (long long)kp.nx * kp.ny * kp.nz))
                        deposit_fixed(qfix + key, to_fixed(qq[w], S));
                }
                key2[w] = key;
                for (int j = 0; j < 3; ++j) g2[j][w] = g[j];
            }
            if (pair_) *reinterpret_cast<uint2*>(keys + i0_) = make_uint2(key2[0], key2[1]);
            else keys[i0_] = key2[0];
            // the el_field entry gathers at the stored grid coordinates; the kick
            // recomputes them from rparticles
            if (!rp)
                for (int j = 0; j < 3; ++j) st_rowf(X + j * nX, i0_, pair_, g2[j][0], g2[j][1]);
        }
        // near-face particles beyond the block's list (degenerate beams only):
        // the FP32-corrected estimate alone, out of the unrolled loop
        while (slow) {
            const int bit = __ffs(slow) - 1;
            slow &= slow - 1;
            const int64_t p_ = pg_ + (bit >> 1) * pstride_;
            const int64_t i = (VEC && p_ < npair_ ? 2 * p_ : (VEC ? n - 1 : p_)) + (bit & 1);
            double T[3][3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) T[a][b] = st->T[a][b];
            double xv[3], e[3];
            xyz_fine32(rp, ld, i, kp, T, st->gamma0, xv);
            for (int j = 0; j < 3; ++j)  // the FP64 form's grid coordinate (k_keys64)
                e[j] = __dsub_rn(div_checked(xv[j], st->steps[j], st->isteps[j]), st->xoff[j]);
            uint32_t key = 0u;
            bad |= !key_of(floor(e[0]) + 1, floor(e[1]) + 1, floor(e[2]) + 1, kp, key);
            keys[i] = key;
            if (qfix && SC_IDX_OK(st, 11, key, (long long)kp.nx * kp.ny * kp.nz))
                deposit_fixed(qfix + key, to_fixed(q[i], S));
        }
    }
    // the listed particles: key from the FP64 coordinates and the deposit;
    // one per thread, so the block waits for one slow FP64 evaluation
    // instead of each warp stalling on its own
    __syncthreads();
    const int nf = s_nfine < KEYS_FINE ? s_nfine : KEYS_FINE;
    for (int e = threadIdx.x; e < nf; e += blockDim.x) {
        const int64_t i = s_fine[e];
        uint32_t key;
        float gf[3];
        bad |= !key_fine(rp, ld, i, kp, st, key, gf);
        keys[i] = key;
        if (qfix && SC_IDX_OK(st, 13, key, (long long)kp.nx * kp.ny * kp.nz))
            deposit_fixed(qfix + key, to_fixed(q[i], S));
    }
    if (bad) atomicCAS(&st->status, SC_OK, SC_ERR_NONFINITE);
}

template <bool VEC>
__global__ void __launch_bounds__(PT, 4) k_keys32(float* __restrict__ X, uint32_t* __restrict__ keys,
                                                  const double* __restrict__ rp, const double* __restrict__ q,
                                                  unsigned long long* __restrict__ qfix, KickParams kp, ScState* st) {
    pdl_wait();
    keys32_body<VEC>(X, keys, rp, q, qfix, kp, st, hw_vblk());
}

// ---------------------------------------------------------------------------
// trilinear gather, scipy.ndimage.map_coordinates(order=1, mode='constant')
// semantics: a sample outside [0, n-1] in any axis is 0
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R trilerp(const R* __restrict__ F, int nx, int ny, int nz, R c0, R c1, R c2) {
    int i, j, k;
    if constexpr (sizeof(R) == 8) {
        if (!in_range64(c0, nx - 1) || !in_range64(c1, ny - 1) || !in_range64(c2, nz - 1)) return 0;
        i = floor_nonneg64(c0);
        j = floor_nonneg64(c1);
        k = floor_nonneg64(c2);
    } else {
        if (!(c0 >= 0) || !(c1 >= 0) || !(c2 >= 0) || c0 > nx - 1 || c1 > ny - 1 || c2 > nz - 1) return 0;
        i = (int)floor(c0);
        j = (int)floor(c1);
        k = (int)floor(c2);
    }
    if (i > nx - 2) i = nx - 2;
    if (j > ny - 2) j = ny - 2;
    if (k > nz - 2) k = nz - 2;
    const R tx = c0 - i, ty = c1 - j, tz = c2 - k;
    const R wx[2] = {1 - tx, tx}, wy[2] = {1 - ty, ty}, wz[2] = {1 - tz, tz};
    const R* b = F + ((size_t)i * ny + j) * nz + k;
    R acc = 0;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const R f = b[((size_t)a * ny + bb) * nz + cc];
                if (sizeof(R) == 8)
                    acc = (R)__dadd_rn((double)acc, __dmul_rn(__dmul_rn(__dmul_rn((double)f, (double)wx[a]), (double)wy[bb]), (double)wz[cc]));
                else
                    acc += f * wx[a] * wy[bb] * wz[cc];
            }
    return acc;
}

template <typename R>
__device__ __forceinline__ void gather3(const R* ex, const R* ey, const R* ez, int nx, int ny, int nz, R X0, R X1,
                                        R X2, R& e0, R& e1, R& e2) {
    const R h = (R)0.5;
    e0 = trilerp<R>(ex, nx, ny, nz, X0, X1 + h, X2 + h);
    e1 = trilerp<R>(ey, nx, ny, nz, X0 + h, X1, X2 + h);
    e2 = trilerp<R>(ez, nx, ny, nz, X0 + h, X1 + h, X2);
}

// trilinear sample from the FP32 gather octs (one 32-byte load)
__device__ __forceinline__ float trilerp_o(const float* __restrict__ O, int nx, int ny, int nz, float c0, float c1,
                                           float c2) {
    if (!(c0 >= 0.f) || !(c1 >= 0.f) || !(c2 >= 0.f) || c0 > (float)(nx - 1) || c1 > (float)(ny - 1) ||
        c2 > (float)(nz - 1))
        return 0.f;
    int i = (int)c0, j = (int)c1, k = (int)c2;
    if (i > nx - 2) i = nx - 2;
    if (j > ny - 2) j = ny - 2;
    if (k > nz - 2) k = nz - 2;
    const float tx = c0 - (float)i, ty = c1 - (float)j, tz = c2 - (float)k;
    const float* p = O + 8 * ((i * ny + j) * nz + k);  // < 2^31: meshes have at most 256^3 cells
    float o[8];
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3]), "=f"(o[4]), "=f"(o[5]), "=f"(o[6]), "=f"(o[7])
        : "l"(p));
    const float ya = (1.f - ty) * ((1.f - tz) * o[0] + tz * o[1]) + ty * ((1.f - tz) * o[2] + tz * o[3]);
    const float yb = (1.f - ty) * ((1.f - tz) * o[4] + tz * o[5]) + ty * ((1.f - tz) * o[6] + tz * o[7]);
    return (1.f - tx) * ya + tx * yb;
}

__device__ __forceinline__ void gather3o(const float* ox, const float* oy, const float* oz, int nx, int ny, int nz,
                                         float X0, float X1, float X2, float& e0, float& e1, float& e2) {
    e0 = trilerp_o(ox, nx, ny, nz, X0, X1 + 0.5f, X2 + 0.5f);
    e1 = trilerp_o(oy, nx, ny, nz, X0 + 0.5f, X1, X2 + 0.5f);
    e2 = trilerp_o(oz, nx, ny, nz, X0 + 0.5f, X1 + 0.5f, X2);
}

// rec != nullptr (the record-field mode): the field samples before the gamma0
// factor go to rec[i], rec[nX + i], rec[2 nX + i] (rec may be X itself: each
// thread writes only the entries it has read)
__global__ void __launch_bounds__(PT) k_kick64(double* __restrict__ rp, const double* __restrict__ xp,
                                               const double* X, const double* __restrict__ ex,
                                               const double* __restrict__ ey, const double* __restrict__ ez,
                                               KickParams kp, const ScState* st, double* rec) {
    pdl_wait();
    if (st->status) return;
    const int64_t n = kp.n, ld = kp.ld;
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = st->T[i][j];
    const double g0 = st->gamma0, kxy = st->kxy, kz = st->kz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double e0, e1, e2;
        gather3<double>(ex, ey, ez, kp.nx, kp.ny, kp.nz, X[i], X[kp.nX + i], X[2 * kp.nX + i], e0, e1, e2);
        if (rec) {
            rec[i] = e0;
            rec[kp.nX + i] = e1;
            rec[2 * kp.nX + i] = e2;
        }
        e0 = __dmul_rn(e0, g0);
        e1 = __dmul_rn(e1, g0);
        const double p0 = xp[3 * n + i], p1 = xp[4 * n + i], p2 = xp[5 * n + i];
        double pr[3];
        for (int j = 0; j < 3; ++j) pr[j] = dot3_blas(p0, p1, p2, T[0][j], T[1][j], T[2][j]);
        pr[0] = __dadd_rn(pr[0], __dmul_rn(kxy, e0));
        pr[1] = __dadd_rn(pr[1], __dmul_rn(kxy, e1));
        pr[2] = __dadd_rn(pr[2], __dmul_rn(kz, e2));
        double pn[3];
        for (int k = 0; k < 3; ++k) pn[k] = dot3_blas(pr[0], pr[1], pr[2], T[k][0], T[k][1], T[k][2]);
        const double pos[3] = {xp[i], xp[n + i], xp[2 * n + i]};
        double r[6];
        cart_to_mad64(pos, pn, kp, r);
#pragma unroll
        for (int k = 0; k < 6; ++k) rp[k * ld + i] = r[k];
    }
}

// per-kick constants of the FP32 gather + kick, loaded once per thread
struct Kick32C {
    float T[3][3];
    float kxyg, kz, ipref, m2;
    float isf[3], of[3];  // 1/steps (times gamma0 along z), X_off
    const float *ox, *oy, *oz;
};
__device__ __forceinline__ Kick32C kick32_const(const ScState* st, const KickParams& kp, const float* ox,
                                                const float* oy, const float* oz) {
    Kick32C c;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) c.T[i][j] = st->Tf[i][j];
    c.kxyg = st->kxyf * st->g0f;
    c.kz = st->kzf;
    c.ipref = kp.ipref_f;
    c.m2 = kp.m2_f;
    for (int j = 0; j < 3; ++j) {
        c.isf[j] = st->istepsf[j];
        c.of[j] = st->xofff[j];
    }
    c.isf[2] *= st->g0f;
    c.ox = ox;
    c.oy = oy;
    c.oz = oz;
    return c;
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }

// Trilinear sample coordinate along one axis of length n (map_coordinates
// order=1, mode='constant'): valid iff 0 <= c <= n-1; base cell min(floor c,
// n-2) and weight c - base.
struct AxisW {
    int i;
    float t;
    bool ok;
};
// The base cell is clamped into [0, n-2] whether or not the sample is valid,
// so that the oct load below is always in bounds and needs no branch.
__device__ __forceinline__ AxisW axis_w(float c, int n) {
    AxisW a;
    a.ok = c >= 0.f && c <= (float)(n - 1);
    int i = (int)c;
    i = i > n - 2 ? n - 2 : i;
    a.i = i < 0 ? 0 : i;
    a.t = c - (float)a.i;
    return a;
}
// one staggered field component from its octs at (ax, ay, az); outside the
// mesh the (in-bounds) load is made and its sample replaced by 0
__device__ __forceinline__ float oct_sample(const float* __restrict__ O, const AxisW& ax, const AxisW& ay,
                                            const AxisW& az, int ny, int nz) {
    const float* p = O + 8 * ((ax.i * ny + ay.i) * nz + az.i);  // < 2^31: meshes have at most 256^3 cells
    float o[8];
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3]), "=f"(o[4]), "=f"(o[5]), "=f"(o[6]), "=f"(o[7])
        : "l"(p));
    const float y0 = lerpf(lerpf(o[0], o[1], az.t), lerpf(o[2], o[3], az.t), ay.t);
    const float y1 = lerpf(lerpf(o[4], o[5], az.t), lerpf(o[6], o[7], az.t), ay.t);
    const float v = lerpf(y0, y1, ax.t);
    return (ax.ok && ay.ok && az.ok) ? v : 0.f;
}

// FP32 gather + kick of one particle, r = its six float64 coordinates,
// updated in place.  The momenta, the rotated grid coordinates and the kick
// are recomputed from r in FP32 with fused multiply-adds and the hardware's
// approximate reciprocal and square root, so the kick reads nothing per
// particle but rparticles.  (The NGP keys, which must equal the FP64 form's,
// are decided by the keys kernel alone; the gather only needs the grid
// coordinates to FP32 accuracy.)  The conversions are branch-free inline
// forms (d2f_kick, f2d_exact): with range-checked forms and out-of-line
// fallbacks the kick kernel, at its 80-register limit, ran 15% slower.
// The kick of one particle as six FP32 increments of its MAD coordinates
// (x, x', y, y', tau, delta), from the coordinates rounded to FP32 (f).
// rec != nullptr (the record-field mode): the three field samples, the
// trilinear gathers of Ex, Ey, Ez at the particle before the gamma0 factor
// (sc.py:201-204), are stored at rec[0], rec[nX], rec[2 nX].
__device__ __forceinline__ void kick_inc(const float (&f)[6], const Kick32C& C, const KickParams& kp,
                                         float (&inc)[6], float* rec = nullptr) {
    float px, py, pz, E;
    mom32(f[1], f[3], f[5], kp, px, py, pz, E);
    // lab position, rotated and scaled to the grid
    const float tau = f[4];
    const float iE = rcpf(E);
    float l[3];
    lab32(f[0], f[2], tau, px, py, pz, E, kp, l);
    float X[3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
        X[j] = fmaf(fmaf(l[0], C.T[0][j], fmaf(l[1], C.T[1][j], l[2] * C.T[2][j])), C.isf[j], -C.of[j]);
    // staggered trilinear gather (sc.py:201-204): each component is sampled
    // at +0.5 on the two axes it is not differentiated along
    const AxisW a0 = axis_w(X[0], kp.nx), a1 = axis_w(X[1], kp.ny), a2 = axis_w(X[2], kp.nz);
    const AxisW b0 = axis_w(X[0] + 0.5f, kp.nx), b1 = axis_w(X[1] + 0.5f, kp.ny), b2 = axis_w(X[2] + 0.5f, kp.nz);
    const float e0 = oct_sample(C.ox, a0, b1, b2, kp.ny, kp.nz);
    const float e1 = oct_sample(C.oy, b0, a1, b2, kp.ny, kp.nz);
    const float e2 = oct_sample(C.oz, b0, b1, a2, kp.ny, kp.nz);
    if (rec) {
        rec[0] = e0;
        rec[kp.nX] = e1;
        rec[2 * kp.nX] = e2;
    }
    // kick in the beam frame, rotated back to the lab (sc.py:244-250)
    const float d0 = C.kxyg * e0, d1 = C.kxyg * e1, d2 = C.kz * e2;
    const float dpx = fmaf(C.T[0][0], d0, fmaf(C.T[0][1], d1, C.T[0][2] * d2));
    const float dpy = fmaf(C.T[1][0], d0, fmaf(C.T[1][1], d1, C.T[1][2] * d2));
    const float dpz = fmaf(C.T[2][0], d0, fmaf(C.T[2][1], d1, C.T[2][2] * d2));
    const float pxn = px + dpx, pyn = py + dpy, pzn = pz + dpz;
    const float En = sqrtf_fast(fmaf(pxn, pxn, fmaf(pyn, pyn, fmaf(pzn, pzn, C.m2))));
    const float iEn = rcpf(En);
    const float pdp = fmaf(px, dpx, fmaf(py, dpy, pz * dpz));
    const float dp2 = fmaf(dpx, dpx, fmaf(dpy, dpy, dpz * dpz));
    const float dE = fmaf(2.0f, pdp, dp2) * rcpf(E + En);
    // pz E' - pz' E without cancellation (it is suppressed by 1/gamma^2):
    //   = [pz^2 dT - dpz (pz + pz') (m^2 + pT^2)] / (pz E' + pz' E),
    //   dT = |pT'|^2 - |pT|^2
    const float pT2 = fmaf(px, px, py * py);
    const float dT = fmaf(2.0f, fmaf(px, dpx, py * dpy), fmaf(dpx, dpx, dpy * dpy));
    const float fz = fmaf(pz * pz, dT, -dpz * (pz + pzn) * (C.m2 + pT2)) * rcpf(fmaf(pz, En, pzn * E));
    const float dtau = tau * fz * iE * rcpf(pzn);
    const float iEE = iE * iEn;
    // new MAD coordinates as increments (coord_transform.py:16-54)
    inc[0] = fmaf(tau * fmaf(dpx, E, -px * dE), iEE, pxn * iEn * dtau);
    inc[1] = dpx * C.ipref;
    inc[2] = fmaf(tau * fmaf(dpy, E, -py * dE), iEE, pyn * iEn * dtau);
    inc[3] = dpy * C.ipref;
    inc[4] = dtau;
    inc[5] = dE * C.ipref;
}

// FP32 gather + kick of one particle, r = its six float64 coordinates,
// updated in place.  The momenta, the rotated grid coordinates and the kick
// are recomputed from r in FP32 with fused multiply-adds and the hardware's
// approximate reciprocal and square root, so the kick reads nothing per
// particle but rparticles.  (The NGP keys, which must equal the FP64 form's,
// are decided by the keys kernel alone; the gather only needs the grid
// coordinates to FP32 accuracy.)  The conversions are branch-free inline
// forms (d2f_kick, f2d_exact): with range-checked forms and out-of-line
// fallbacks the kick kernel, at its 80-register limit, ran 15% slower.  The
// only FP64 arithmetic is the six additions into the float64 coordinates.
__device__ __forceinline__ void kick_one(double (&r)[6], const Kick32C& C, const KickParams& kp,
                                         float* rec = nullptr) {
    float f[6], inc[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) f[k] = d2f_kick(r[k]);
    kick_inc(f, C, kp, inc, rec);
#pragma unroll
    for (int k = 0; k < 6; ++k) r[k] += f2d_exact(inc[k]);
}

// one double from shared memory, read where it stands in the program (not
// merged with an earlier read of the same word, so it holds no register
// across the code between)
__device__ __forceinline__ double ld_shared_f64(const double* p) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(smem_u32(p)));
    return v;
}

// Gather + kick with direct row accesses: each thread takes G consecutive
// particles with one 32-byte (G = 4) or 16-byte (G = 2) access per row.
template <int G, bool REC = false>
__device__ __forceinline__ void kick32_body(double* __restrict__ rp, const float* __restrict__ ox,
                                            const float* __restrict__ oy, const float* __restrict__ oz,
                                            const KickParams& kp, const ScState* st, VBlk vb,
                                            float* __restrict__ rec = nullptr) {
    if (st->status) return;
    const int64_t n = kp.n, ld = kp.ld;
    const Kick32C C = kick32_const(st, kp, ox, oy, oz);
    GROUP_LOOP_BEGIN(n, G)
    double r[6][G];
#pragma unroll
    for (int k = 0; k < 6; ++k) ld_rows<G>(rp + k * ld, i0_, full_, r[k]);
#pragma unroll
    for (int w = 0; w < G; ++w) {
        if (w >= W_) break;
        double x[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = r[k][w];
        kick_one(x, C, kp, REC ? rec + i0_ + w : nullptr);
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k][w] = x[k];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) st_rows<G>(rp + k * ld, i0_, full_, r[k]);
    GROUP_LOOP_END
}

// Gather + kick with the rows staged through shared memory by bulk (TMA)
// copies.  A block walks its tiles of TILE particles (its first tile is its
// block index, every further one is claimed at run time); STAGES tile
// buffers of the six rows rotate: while the block kicks one tile, the loads
// of the next STAGES - 1 are in flight, so the HBM stream does not wait for
// the gathers.  Each of the TILE / PPT threads kicks PPT adjacent particles of
// a tile in place in shared memory, and one bulk store per row writes the
// tile back.  Rows must be 16-byte aligned with an even stride.  A tile's
// copies cover its first (count & ~1) particles; an odd last particle of the
// beam is read and written directly.  Every particle's arithmetic is
// kick_one whatever the tiling, so all tilings give the same bits.
template <int TILE, int STAGES, int PPT>
struct KickTiling {
    static_assert(PPT == 1 || PPT == 2, "one or two particles per thread");
    static constexpr int threads = TILE / PPT;
    static constexpr size_t smem = (size_t)STAGES * 6 * TILE * sizeof(double) + STAGES * sizeof(uint64_t);
};

template <int TILE, int STAGES, int PPT>
__device__ __forceinline__ void kick32_tma_body(double* __restrict__ rp, const float* __restrict__ ox,
                                                const float* __restrict__ oy, const float* __restrict__ oz,
                                                const KickParams& kp, ScState* st, VBlk vb) {
    extern __shared__ __align__(128) unsigned char smraw[];
    if (__syncthreads_or(st->status != SC_OK)) return;
    double* buf = reinterpret_cast<double*>(smraw);  // [STAGES][6][TILE]
    uint64_t* bar = reinterpret_cast<uint64_t*>(buf + STAGES * 6 * TILE);
    const int64_t n = kp.n, ld = kp.ld;
    const int64_t ntile = (n + TILE - 1) / TILE;
    const bool lead = threadIdx.x == 0;
    // Tiles are handed out at run time: a block's first tile is its index,
    // each further one is claimed from the kick's tile counter when its
    // loads are issued, so blocks on faster SMs take more tiles and the
    // blocks finish together.  s_tile[s] is the tile in buffer s; a tile
    // index >= ntile marks the end.  (The tiles are independent: which block
    // kicks a particle does not change its result.)
    __shared__ int64_t s_tile[STAGES];
    if (lead) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&bar[s], 1);
        mbar_init_fence();
    }
    __syncthreads();
    auto tile_start = [&](int64_t g) { return g * (int64_t)TILE; };
    auto tile_count = [&](int64_t g) {
        const int64_t c = n - tile_start(g);
        return (int)(c < TILE ? c : TILE);
    };
    auto claim = [&]() { return (int64_t)vb.nx + (int64_t)atomicAdd(&st->kick_next, 1u); };
    auto issue = [&](int64_t u, int64_t g) {  // lead thread: tile g as the block's u-th, into buffer u % STAGES
        const int s = (int)(u % STAGES);
        s_tile[s] = g;
        if (g >= ntile) return;
        const int64_t i0 = tile_start(g);
        const unsigned bytes = (unsigned)(tile_count(g) & ~1) * 8u;
        mbar_arrive_expect_tx(&bar[s], 6u * bytes);
        if (bytes)
            for (int k = 0; k < 6; ++k) bulk_load(buf + (s * 6 + k) * TILE, rp + k * ld + i0, bytes, &bar[s]);
    };
    int64_t issued = 0;  // lead: tiles issued (the end marker included)
    bool more = true;    // lead: the last claim was a tile
    if (lead)
        for (int u = 0; u < STAGES && more; ++u) {
            const int64_t g = u == 0 ? (int64_t)vb.x : claim();
            issue(issued++, g);
            more = g < ntile;
        }
    __syncthreads();
    const Kick32C C = kick32_const(st, kp, ox, oy, oz);
    int64_t t = 0;
    bool failed = false;
    for (;; ++t) {
        const int s = (int)(t % STAGES);
        const int64_t g = s_tile[s];
        if (g >= ntile) break;  // the same in every thread
        const int64_t i0 = tile_start(g);
        const int cnt = tile_count(g), staged = cnt & ~1;
        const bool ok = mbar_wait(&bar[s], (unsigned)((t / STAGES) & 1), kp.wait_limit[2]);
        double* B = buf + s * 6 * TILE;
        const int j = PPT * threadIdx.x;
        if (PPT == 2 && j + 1 < staged) {  // both particles staged
            // the FP32 coordinates for the kicks; the float64 values are read
            // again for the additions, so they hold no registers meanwhile
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                float f[6], inc[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) f[k] = d2f_kick(ld_shared_f64(B + k * TILE + j + w));
                kick_inc(f, C, kp, inc);
#pragma unroll
                for (int k = 0; k < 6; ++k) B[k * TILE + j + w] = ld_shared_f64(B + k * TILE + j + w) + f2d_exact(inc[k]);
            }
        } else if (PPT == 1 && j < staged) {
            float f[6], inc[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) f[k] = d2f_kick(ld_shared_f64(B + k * TILE + j));
            kick_inc(f, C, kp, inc);
#pragma unroll
            for (int k = 0; k < 6; ++k) B[k * TILE + j] = ld_shared_f64(B + k * TILE + j) + f2d_exact(inc[k]);
        } else if (j < cnt && ok) {  // the odd last particle of the beam (j == staged): read and written directly
            double r[6];
            for (int k = 0; k < 6; ++k) r[k] = rp[k * ld + i0 + j];
            kick_one(r, C, kp);
            for (int k = 0; k < 6; ++k) rp[k * ld + i0 + j] = r[k];
        }
        fence_async_smem();
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        if (lead) {
            if (staged)
                for (int k = 0; k < 6; ++k) bulk_store(rp + k * ld + i0, B + k * TILE, (unsigned)staged * 8u);
            bulk_commit();
            // refill the previous tile's buffer once its store has read it
            if (t >= 1 && more) {
                bulk_wait_read<1>();
                const int64_t g2 = claim();
                issue(issued++, g2);
                more = g2 < ntile;
            }
        }
        // the buffer refilled here is read STAGES - 1 iterations on, after
        // the barriers of the iterations between; with two buffers that is
        // the next iteration, so a barrier publishes the lead's s_tile first
        if constexpr (STAGES < 3) __syncthreads();
    }
    if (lead) {
        if (failed) {
            atomicCAS(&st->status, SC_OK, SC_ERR_TIMEOUT);
            for (int64_t u = t; u < issued; ++u)  // loads still in flight must land before the block exits
                if (s_tile[u % STAGES] < ntile) mbar_wait(&bar[u % STAGES], (unsigned)((u / STAGES) & 1));
        }
        bulk_wait_all();
    }
}

// Gather + kick without block barriers: each thread streams its particles
// through a private ring of STAGES slots in shared memory (the six doubles of
// one particle per slot, [STAGES][6][threads] so that a warp's lanes touch
// consecutive words) with per-thread asynchronous copies, and waits only for
// its own copies -- so a warp whose gathers return late holds up no other
// warp.  Work goes in chunks of 32 consecutive particles (one per lane) that
// warps take in turn: a warp's first chunk is its index in the grid, each
// further one is claimed from the kick's counter when its copies are issued,
// STAGES - 1 chunks ahead of the one being kicked.  Results are stored
// directly (each warp writes 256 contiguous bytes per row).  Any row stride
// works (the copies are 8 bytes).  Every particle's arithmetic is kick_one,
// so this gives the same bits as every other tiling.
template <int STAGES>
__device__ __forceinline__ void kick32_async_body(double* __restrict__ rp, const float* __restrict__ ox,
                                                  const float* __restrict__ oy, const float* __restrict__ oz,
                                                  const KickParams& kp, ScState* st, VBlk vb,
                                                  float* __restrict__ rec = nullptr) {
    extern __shared__ __align__(128) unsigned char smraw[];
    if (st->status != SC_OK) return;  // read by every thread; the frame set it before this launch
    double* ring = reinterpret_cast<double*>(smraw);  // [STAGES][6][blockDim.x]
    const int nt = (int)blockDim.x, lane = (int)(threadIdx.x & 31);
    const int64_t n = kp.n, ld = kp.ld;
    const int64_t nchunk = (n + 31) / 32;
    const int64_t wpb = nt / 32;
    // chunks are handed out in units of CLAIM consecutive chunks: one atomic
    // per unit; a warp's first unit is its index in the grid
    constexpr int CLAIM = 4;
    const int64_t nwarps = (int64_t)vb.nx * wpb;
    int64_t unit = (int64_t)vb.x * wpb + (threadIdx.x >> 5);
    int in_unit = 0;
    auto claim = [&]() -> int64_t {
        if (in_unit == CLAIM) {
            unsigned c = 0;
            if (lane == 0) c = atomicAdd(&st->kick_next, 1u);
            unit = nwarps + (int64_t)__shfl_sync(FULL, c, 0);
            in_unit = 0;
        }
        const int64_t c = unit * CLAIM + in_unit++;
        return c < nchunk ? c : nchunk;
    };
    auto issue = [&](int s, int64_t c) {  // this lane's particle of chunk c into slot s
        const int64_t i = c * 32 + lane;
        if (c < nchunk && i < n) {
            double* slot = ring + (size_t)s * 6 * nt + threadIdx.x;
#pragma unroll
            for (int k = 0; k < 6; ++k) async_copy8(slot + k * nt, rp + k * ld + i, 8u);
        }
        async_commit();  // one group per slot, empty or not, so that the group count stays in step
    };
    const Kick32C C = kick32_const(st, kp, ox, oy, oz);
    int64_t chunk[STAGES];
    bool more = true;  // the last claim was a chunk (the same in every lane of the warp)
#pragma unroll
    for (int s = 0; s < STAGES; ++s) {
        chunk[s] = !more ? nchunk : claim();
        more = chunk[s] < nchunk;
        issue(s, chunk[s]);
    }
    for (int64_t t = 0;; ++t) {
        const int s = (int)(t % STAGES);
        int64_t c = 0;
#pragma unroll
        for (int u = 0; u < STAGES; ++u)
            if (u == s) c = chunk[u];
        if (c >= nchunk) break;
        async_wait<STAGES - 1>();  // this thread's copies of slot s have landed
        const int64_t i = c * 32 + lane;
        if (i < n) {
            // the coordinates in FP32 for the kick; the float64 values are read
            // again for the additions, so they hold no registers meanwhile
            const double* slot = ring + (size_t)s * 6 * nt + threadIdx.x;
            float f[6], inc[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) f[k] = d2f_kick(ld_shared_f64(slot + k * nt));
            kick_inc(f, C, kp, inc, rec ? rec + i : nullptr);
#pragma unroll
            for (int k = 0; k < 6; ++k) rp[k * ld + i] = ld_shared_f64(slot + k * nt) + f2d_exact(inc[k]);
        }
        const int64_t nc = more ? claim() : nchunk;
        more = nc < nchunk;
#pragma unroll
        for (int u = 0; u < STAGES; ++u)
            if (u == s) chunk[u] = nc;
        issue(s, nc);
    }
    async_wait<0>();
}

// The kick's tilings: (tile, tile buffers, particles per thread, blocks per
// SM the kernel is compiled for).  Variant 0 is the default; a plan's
// kick_variant selects another (autotuned per mesh and particle count).
#define SC_KICK_VARIANTS(X)  \
    X(0, 512, 3, 2, 3)       \
    X(1, 512, 2, 2, 4)       \
    X(2, 256, 3, 1, 4)       \
    X(3, 256, 2, 1, 5)       \
    X(4, 128, 4, 1, 8)       \
    X(5, 256, 4, 1, 3)       \
    X(6, 512, 3, 1, 2)       \
    X(7, 1024, 3, 1, 1)      \
    X(8, 256, 3, 1, 5)
// the barrier-free tilings (kick32_async_body, 256 threads): (slots per thread, blocks per SM)
#define SC_KICK_ASYNC_VARIANTS(X) \
    X(9, 3, 5)                    \
    X(10, 4, 4)                   \
    X(11, 2, 6)                   \
    X(12, 6, 3)                   \
    X(13, 3, 4)
// more bulk-copy tilings (indices after the barrier-free ones)
#define SC_KICK_VARIANTS_B(X) \
    X(14, 256, 3, 1, 6)       \
    X(15, 256, 2, 1, 6)       \
    X(16, 128, 4, 1, 6)       \
    X(17, 128, 3, 1, 6)       \
    X(18, 128, 6, 1, 6)       \
    X(19, 64, 4, 1, 12)       \
    X(20, 64, 6, 1, 12)

// the default: 128-particle tiles of one particle per thread, four tile
// buffers, six blocks of 128 threads per SM (the same 80 registers as the
// 256-particle tilings): measured fastest on 48^3 to 128x128x256 meshes from
// 200k particles up -- the half-size tiles halve the tail of the kernel (a
// block's last tile) and a slow warp holds four warps at the barrier instead
// of eight (2M / 64^3: 57.3 -> 55.2 us; 10M / 128x128x256: 303 -> 279 us
// with the 3-buffer form)
constexpr int kDefaultKickVariant = 16;
constexpr int kBatchKickVariant = 13;  // the batched kick's tiling (launch_batch_particles)

template <int TILE, int STAGES, int PPT, int MINB>
__global__ void __launch_bounds__(KickTiling<TILE, STAGES, PPT>::threads, MINB)
    k_kick32_tma(double* __restrict__ rp, const float* __restrict__ ox, const float* __restrict__ oy,
                 const float* __restrict__ oz, KickParams kp, ScState* st) {
    pdl_wait();
    kick32_tma_body<TILE, STAGES, PPT>(rp, ox, oy, oz, kp, st, hw_vblk());
}

template <int STAGES, int MINB>
__global__ void __launch_bounds__(PT, MINB)
    k_kick32_async(double* __restrict__ rp, const float* __restrict__ ox, const float* __restrict__ oy,
                   const float* __restrict__ oz, KickParams kp, ScState* st) {
    pdl_wait();
    kick32_async_body<STAGES>(rp, ox, oy, oz, kp, st, hw_vblk());
}

constexpr int KICK_MIN_BLOCKS = 3;  // blocks per SM of the direct-access kick kernels

// rec != nullptr only in the record-field mode (REC)
template <int G, bool REC = false>
__global__ void __launch_bounds__(PT, KICK_MIN_BLOCKS) k_kick32(double* __restrict__ rp, const float* __restrict__ ox,
                                                                const float* __restrict__ oy,
                                                                const float* __restrict__ oz, KickParams kp,
                                                                const ScState* st, float* __restrict__ rec) {
    pdl_wait();
    kick32_body<G, REC>(rp, ox, oy, oz, kp, st, hw_vblk(), rec);
}

// particles per row access the kick can use: 4 with 32-byte aligned rows and
// a row stride that is a multiple of 4, 2 with 16-byte alignment and an even
// stride, else 1
__host__ __device__ __forceinline__ int kick_group(const double* rp, int64_t ld) {
    if ((uintptr_t)rp % 32 == 0 && ld % 4 == 0) return 4;
    if ((uintptr_t)rp % 16 == 0 && ld % 2 == 0) return 2;
    return 1;
}

template <typename R>
__global__ void __launch_bounds__(PT) k_gather_xyz(const R* __restrict__ X, const R* __restrict__ ex,
                                                   const R* __restrict__ ey, const R* __restrict__ ez,
                                                   double* __restrict__ out, KickParams kp, const ScState* st) {
    pdl_wait();
    if (st->status) return;
    const int64_t n = kp.n, nX = kp.nX;
    const double g0 = st->gamma0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R e0, e1, e2;
        if (sizeof(R) == 4)
            gather3o(reinterpret_cast<const float*>(ex), reinterpret_cast<const float*>(ey),
                     reinterpret_cast<const float*>(ez), kp.nx, kp.ny, kp.nz, (float)X[i], (float)X[nX + i],
                     (float)X[2 * nX + i], *reinterpret_cast<float*>(&e0), *reinterpret_cast<float*>(&e1),
                     *reinterpret_cast<float*>(&e2));
        else
            gather3<R>(ex, ey, ez, kp.nx, kp.ny, kp.nz, X[i], X[nX + i], X[2 * nX + i], e0, e1, e2);
        out[3 * i] = __dmul_rn((double)e0, g0);
        out[3 * i + 1] = __dmul_rn((double)e1, g0);
        out[3 * i + 2] = (double)e2;
    }
}

// ---------------------------------------------------------------------------
// batched particle stages: one launch over every beam of a batch
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(PT, 4) kb_frame32(const BatchBeam* __restrict__ beams,
                                                    const int* __restrict__ start, int nb) {
    pdl_wait();
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    const VBlk vb = batch_vblk(start, b, B.gx[BS_PART], 1);
    ScState* st = reinterpret_cast<ScState*>(B.ws + B.L.state);
    double* part = reinterpret_cast<double*>(B.ws + B.L.part_frame);
    unsigned long long* qz = reinterpret_cast<unsigned long long*>(B.ws + B.L.qfix);
    const int64_t nc = (int64_t)B.p.nx * B.p.ny * B.p.nz;
    if (B.vec_rp) frame32_tma_body(B.rp, B.kp, part, st, qz, nc, vb);
    else frame32_body<false>(B.rp, B.kp, part, st, qz, nc, vb);
}

__global__ void __launch_bounds__(PT, 3) kb_extent32(const BatchBeam* __restrict__ beams,
                                                     const int* __restrict__ start, int nb) {
    pdl_wait();
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    const VBlk vb = batch_vblk(start, b, B.gx[BS_PART], 1);
    ScState* st = reinterpret_cast<ScState*>(B.ws + B.L.state);
    float* X = reinterpret_cast<float*>(B.ws + B.L.X);
    double* part = reinterpret_cast<double*>(B.ws + B.L.part_ext);
    if (B.vec_rpq) extent32_tma_body(B.rp, B.q, B.kp, X, part, st, vb);
    else extent32_body<false>(B.rp, B.q, B.kp, X, part, st, vb);
}

__global__ void __launch_bounds__(PT, 4) kb_keys32(const BatchBeam* __restrict__ beams,
                                                   const int* __restrict__ start, int nb) {
    pdl_wait();
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    const VBlk vb = batch_vblk(start, b, B.gx[BS_PART], 1);
    ScState* st = reinterpret_cast<ScState*>(B.ws + B.L.state);
    float* X = reinterpret_cast<float*>(B.ws + B.L.X);
    uint32_t* keys = reinterpret_cast<uint32_t*>(B.ws + B.L.keys);
    unsigned long long* qfix = reinterpret_cast<unsigned long long*>(B.ws + B.L.qfix);
    if ((uintptr_t)B.q % 16 == 0) keys32_body<true>(X, keys, B.rp, B.q, qfix, B.kp, st, vb);
    else keys32_body<false>(X, keys, B.rp, B.q, qfix, B.kp, st, vb);
}

template <int STAGES, int MINB>
__global__ void __launch_bounds__(PT, MINB) kb_kick32_async(const BatchBeam* __restrict__ beams,
                                                            const int* __restrict__ start, int nb) {
    pdl_wait();
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    const VBlk vb = batch_vblk(start, b, B.gx[BS_PART], 1);
    ScState* st = reinterpret_cast<ScState*>(B.ws + B.L.state);
    kick32_async_body<STAGES>(B.rp, reinterpret_cast<const float*>(B.ws + B.L.exq),
                              reinterpret_cast<const float*>(B.ws + B.L.eyq),
                              reinterpret_cast<const float*>(B.ws + B.L.ezq), B.kp, st, vb);
}

template <int TILE, int STAGES, int PPT, int MINB>
__global__ void __launch_bounds__(KickTiling<TILE, STAGES, PPT>::threads, MINB)
    kb_kick32(const BatchBeam* __restrict__ beams, const int* __restrict__ start, int nb) {
    pdl_wait();
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    const VBlk vb = batch_vblk(start, b, B.gx[BS_PART], 1);
    ScState* st = reinterpret_cast<ScState*>(B.ws + B.L.state);
    const float* ox = reinterpret_cast<const float*>(B.ws + B.L.exq);
    const float* oy = reinterpret_cast<const float*>(B.ws + B.L.eyq);
    const float* oz = reinterpret_cast<const float*>(B.ws + B.L.ezq);
    if (kick_group(B.rp, B.kp.ld) >= 2) kick32_tma_body<TILE, STAGES, PPT>(B.rp, ox, oy, oz, B.kp, st, vb);
    else kick32_body<1>(B.rp, ox, oy, oz, B.kp, st, vb);  // rows without 16-byte alignment: the direct-access loop
}

// the compiled kick tilings, indexed by a plan's kick_variant
using KickFn = void (*)(double*, const float*, const float*, const float*, KickParams, ScState*);
using KickBatchFn = void (*)(const BatchBeam*, const int*, int);
struct KickVariant {
    KickFn fn;
    KickBatchFn batch_fn;
    int tile, stages, ppt, minb, threads;  // tile 32: a barrier-free tiling (chunks of 32 per warp)
    size_t smem;
    bool any_rows;                         // runs on any row stride (else 16-byte aligned rows, even stride)
};
static const KickVariant kKickVariants[] = {
#define SC_KV(i, T, S, P, M)                                                                                       \
    {k_kick32_tma<T, S, P, M>, kb_kick32<T, S, P, M>, T, S, P, M, KickTiling<T, S, P>::threads,                  \
     KickTiling<T, S, P>::smem, false},
    SC_KICK_VARIANTS(SC_KV)
#define SC_KA(i, S, M) \
    {k_kick32_async<S, M>, kb_kick32_async<S, M>, 32, S, 1, M, PT, (size_t)S * 6 * PT * sizeof(double), true},
    SC_KICK_ASYNC_VARIANTS(SC_KA)
#undef SC_KA
    SC_KICK_VARIANTS_B(SC_KV)
#undef SC_KV
};
constexpr int kNumKickVariants = (int)(sizeof(kKickVariants) / sizeof(kKickVariants[0]));
static_assert(KickTiling<256, 3, 1>::threads == PT, "the 256-particle, one-per-thread tilings have PT threads");
static_assert(kNumKickVariants == SC_KICK_NVARIANTS, "SC_KICK_NVARIANTS must count SC_KICK_VARIANTS");

int default_kick_variant() { return kDefaultKickVariant; }

int kick_variant_info(int v, int* tile, int* stages, int* ppt, int* minb) {
    if (v < 0 || v >= kNumKickVariants) return 0;
    const KickVariant& k = kKickVariants[v];
    *tile = k.tile;
    *stages = k.stages;
    *ppt = k.ppt;
    *minb = k.minb;
    return 1;
}

cudaError_t launch_batch_particles(BatchPartKernel k, const BatchBeam* beams, const int* start, int nb, int blocks,
                                   cudaStream_t s) {
    if (blocks <= 0) return cudaSuccess;
    switch (k) {
        case BP_FRAME: launch(kb_frame32, blocks, PT, FR_SMEM, s, beams, start, nb); break;
        case BP_EXTENT: launch(kb_extent32, blocks, PT, EX_SMEM, s, beams, start, nb); break;
        case BP_KEYS: launch(kb_keys32, blocks, PT, 0, s, beams, start, nb); break;
        case BP_KICK: {
            // the batch's particle blocks (BS_PART, 256 threads) run the
            // barrier-free tiling (3 slots, 4 blocks per SM): measured on the
            // 96-beam batch, kick stage 1.71 -> 1.54 ms against the bulk-copy
            // default (the same bits)
            const KickVariant& v = kKickVariants[kBatchKickVariant];
            launch(v.batch_fn, blocks, v.threads, v.smem, s, beams, start, nb);
            break;
        }
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t prepare_particle_kernels() {
    cudaError_t e;
    for (int v = 0; v < kNumKickVariants; ++v) {
        if ((e = set_smem(kKickVariants[v].fn, kKickVariants[v].smem))) return e;
        if ((e = set_smem(kKickVariants[v].batch_fn, kKickVariants[v].smem))) return e;
    }
    if ((e = set_smem(k_frame32_tma, FR_SMEM))) return e;
    if ((e = set_smem(kb_frame32, FR_SMEM))) return e;
    if ((e = set_smem(k_extent32_tma, EX_SMEM))) return e;
    return set_smem(kb_extent32, EX_SMEM);
}

// 16-byte row accesses need 16-byte aligned rows and an even row stride
static bool vec_ok(const double* rp, int64_t ld, const double* q) {
    return ((uintptr_t)rp % 16 == 0) && (ld % 2 == 0) && (q == nullptr || (uintptr_t)q % 16 == 0);
}

// blocks of the frame, extent and keys stages: one per tile of PT_TILE
// particles, at most three per SM (each walks its tiles with the loads of
// the next one in flight)
static int particle_blocks(const Plan& p, int64_t n) {
    int64_t b = (n + PT_TILE - 1) / PT_TILE;
    const int64_t cap = 3 * (int64_t)p.sm_count;
    if (b > cap) b = cap;
    return (int)(b > 0 ? b : 1);
}

int batch_particle_blocks(const Plan& p, int64_t n) { return particle_blocks(p, n); }

cudaError_t launch_frame(const Plan& p, const Layout& L, char* ws, const KickParams& kp, const double* rp,
                         cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part_frame);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        launch(k_frame64, nb, PT, 0, s, rp, kp, reinterpret_cast<double*>(ws + L.xp), part, st);
    else {
        // the exact deposit's fixed-point grid is zeroed here, so the keys
        // kernel follows the extent kernel without a memset between them
        unsigned long long* qz = p.sorted_deposit ? nullptr : reinterpret_cast<unsigned long long*>(ws + L.qfix);
        const int64_t nz = qz ? (int64_t)p.nx * p.ny * p.nz : 0;
        vec_ok(rp, kp.ld, nullptr) ? launch(k_frame32_tma, nb, PT, FR_SMEM, s, rp, kp, part, st, qz, nz)
                                   : launch(k_frame32<false>, nb, PT, 0, s, rp, kp, part, st, qz, nz);
    }
    return cudaGetLastError();
}

cudaError_t launch_extent(const Plan& p, const Layout& L, char* ws, const KickParams& kp, const double* rp,
                          const double* q, cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part_ext);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        launch(k_extent64, nb, PT, 0, s, reinterpret_cast<const double*>(ws + L.xp), q, kp,
                                     reinterpret_cast<double*>(ws + L.X), part, st);
    else
        vec_ok(rp, kp.ld, q)
            ? launch(k_extent32_tma, nb, PT, EX_SMEM, s, rp, q, kp, reinterpret_cast<float*>(ws + L.X), part, st)
            : launch(k_extent32<false>, nb, PT, 0, s, rp, q, kp, reinterpret_cast<float*>(ws + L.X), part, st);
    return cudaGetLastError();
}

cudaError_t launch_extent_xyz(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double* X,
                              const double* q, double gamma, cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part_ext);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        launch(k_extent_xyz<double>, nb, PT, 0, s, X, q, kp, gamma, reinterpret_cast<double*>(ws + L.X), part, st);
    else
        launch(k_extent_xyz<float>, nb, PT, 0, s, X, q, kp, gamma, reinterpret_cast<float*>(ws + L.X), part, st);
    return cudaGetLastError();
}

cudaError_t launch_set_mesh(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double hx, double hy,
                            double hz, cudaStream_t s) {
    (void)p;
    launch(k_set_mesh, 1, 1, 0, s, reinterpret_cast<ScState*>(ws + L.state), hx, hy, hz, kp);
    return cudaGetLastError();
}

cudaError_t launch_keys(const Plan& p, const Layout& L, char* ws, const KickParams& kp, const double* rp,
                        const double* q, cudaStream_t s, bool qfix_zeroed) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    const int nb = particle_blocks(p, kp.n);
    uint32_t* keys = reinterpret_cast<uint32_t*>(ws + L.keys);
    if (p.prec == SC_FP64)
        launch(k_keys64, nb, PT, 0, s, reinterpret_cast<double*>(ws + L.X), keys, kp, st);
    else
    {
        unsigned long long* qfix = nullptr;
        if (q && !p.sorted_deposit) {
            qfix = reinterpret_cast<unsigned long long*>(ws + L.qfix);
            if (!qfix_zeroed) {
                cudaError_t e = cudaMemsetAsync(qfix, 0, 8 * (size_t)p.nx * p.ny * p.nz, s);
                if (e) return e;
            }
        }
        if (!qfix || (uintptr_t)q % 16 == 0)
            launch(k_keys32<true>, nb, PT, 0, s, reinterpret_cast<float*>(ws + L.X), keys, rp, q, qfix, kp, st);
        else
            launch(k_keys32<false>, nb, PT, 0, s, reinterpret_cast<float*>(ws + L.X), keys, rp, q, qfix, kp, st);
    }
    return cudaGetLastError();
}

cudaError_t launch_gather_kick(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double* rp,
                               cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        launch(k_kick64, nb, PT, 0, s, rp, reinterpret_cast<const double*>(ws + L.xp),
                                   reinterpret_cast<const double*>(ws + L.X), reinterpret_cast<const double*>(ws + L.ex),
                                   reinterpret_cast<const double*>(ws + L.ey), reinterpret_cast<const double*>(ws + L.ez),
                                   kp, st, p.record_field ? reinterpret_cast<double*>(ws + L.X) : nullptr);
    else
    {
        const float* ox = reinterpret_cast<const float*>(ws + L.exq);
        const float* oy = reinterpret_cast<const float*>(ws + L.eyq);
        const float* oz = reinterpret_cast<const float*>(ws + L.ezq);
        const int g = kick_group(rp, kp.ld);
        // one wave of resident blocks, each looping over its tiles or groups
        const KickVariant& v = kKickVariants[p.kick_variant >= 0 && p.kick_variant < kNumKickVariants ? p.kick_variant : 0];
        const bool tiled = g >= 2 || v.any_rows;
        const int minb = tiled ? v.minb : KICK_MIN_BLOCKS;
        const int per_block = v.any_rows ? v.threads : v.tile;  // particles per block per round
        const int64_t units = tiled ? (kp.n + per_block - 1) / per_block : (kp.n + PT - 1) / PT;
        const int64_t kb = units < (int64_t)p.sm_count * minb ? units : (int64_t)p.sm_count * minb;
        const int nbk = (int)(kb > 0 ? kb : 1);
        ScState* stw = reinterpret_cast<ScState*>(ws + L.state);
        if (p.record_field)  // the direct-access loop, storing the field samples in the X rows
            launch(k_kick32<1, true>, nbk, PT, 0, s, rp, ox, oy, oz, kp, st, reinterpret_cast<float*>(ws + L.X));
        else if (tiled) launch(v.fn, nbk, v.threads, v.smem, s, rp, ox, oy, oz, kp, stw);
        else launch(k_kick32<1, false>, nbk, PT, 0, s, rp, ox, oy, oz, kp, st, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_gather_xyz(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double* exyz,
                              cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        launch(k_gather_xyz<double>, nb, PT, 0, s, reinterpret_cast<const double*>(ws + L.X),
                                               reinterpret_cast<const double*>(ws + L.ex),
                                               reinterpret_cast<const double*>(ws + L.ey),
                                               reinterpret_cast<const double*>(ws + L.ez), exyz, kp, st);
    else
        launch(k_gather_xyz<float>, nb, PT, 0, s, reinterpret_cast<const float*>(ws + L.X),
                                              reinterpret_cast<const float*>(ws + L.exq),
                                              reinterpret_cast<const float*>(ws + L.eyq),
                                              reinterpret_cast<const float*>(ws + L.ezq), exyz, kp, st);
    return cudaGetLastError();
}

}  // namespace ocsc
