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
//     dtau = tau (pz dE - E dpz) / (E pz')
//     dx   = tau (dpx E - px dE) / (E E') + (px'/E') dtau      (same for y)
// Reductions are deterministic: a fixed grid, shuffle trees within blocks,
// per-block partials in HBM and a one-block finalize in a fixed order.
#include "sc_common.cuh"

namespace ocsc {

constexpr int PT = 256;  // threads per block of the particle kernels
constexpr unsigned FULL = 0xffffffffu;

// ---------------------------------------------------------------------------
// deterministic block reductions
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sm /* NV*32 */) {
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

template <int NV, bool MAX>
__device__ __forceinline__ void block_minmax(double (&v)[NV], double* sm) {
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

// ---------------------------------------------------------------------------
// FP64 transforms in the reference's operation order
// ---------------------------------------------------------------------------
// xxstg_2_xp_mad (coord_transform.py:57-96)
__device__ __forceinline__ void mad_to_cart64(const double r[6], const KickParams& kp, double xp[6]) {
    const double gamma = __dmul_rn(__dadd_rn(__dmul_rn(kp.betaref, r[5]), 1.0), kp.gamref);
    const double beta = __dsqrt_rn(__dsub_rn(1.0, __drcp_rn(__dmul_rn(gamma, gamma))));
    const double g = __ddiv_rn(__dmul_rn(gamma, beta), kp.grbr);
    const double pz2pref = __dsqrt_rn(__dsub_rn(__dsub_rn(__dmul_rn(g, g), __dmul_rn(r[1], r[1])), __dmul_rn(r[3], r[3])));
    double u0 = __ddiv_rn(r[1], pz2pref), u1 = __ddiv_rn(r[3], pz2pref);
    const double nrm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(u0, u0), __dmul_rn(u1, u1)), 1.0));
    u0 = __ddiv_rn(u0, nrm);
    u1 = __ddiv_rn(u1, nrm);
    const double u2 = __ddiv_rn(1.0, nrm);
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
    const double gamma = __dsqrt_rn(__dadd_rn(1.0, __ddiv_rn(s, kp.m2)));
    const double beta = __dsqrt_rn(__dsub_rn(1.0, __drcp_rn(__dmul_rn(gamma, gamma))));
    const double p0 = __dsqrt_rn(s);
    const double u0 = __ddiv_rn(p[0], p0), u1 = __ddiv_rn(p[1], p0), u2 = __ddiv_rn(p[2], p0);
    const double cdt = __ddiv_rn(-pos[2], __dmul_rn(beta, u2));
    r[0] = __dadd_rn(pos[0], __dmul_rn(__dmul_rn(beta, u0), cdt));
    r[2] = __dadd_rn(pos[1], __dmul_rn(__dmul_rn(beta, u1), cdt));
    r[5] = __ddiv_rn(__dsub_rn(__ddiv_rn(gamma, kp.gamref), 1.0), kp.betaref);
    r[4] = cdt;
    r[1] = __ddiv_rn(p[0], kp.pref);
    r[3] = __ddiv_rn(p[1], kp.pref);
}

// numpy's [N,3]@[3,3] row product: fma(a2,b2, fma(a1,b1, a0*b0))
__device__ __forceinline__ double dot3_blas(double a0, double a1, double a2, double b0, double b1, double b2) {
    return __fma_rn(a2, b2, __fma_rn(a1, b1, __dmul_rn(a0, b0)));
}

// ---------------------------------------------------------------------------
// FP32 forward quantities from the FP64 MAD coordinates
// ---------------------------------------------------------------------------
struct F32Consts {
    float gamref, betaref, grbr, pref, m, m2;
};
__device__ __forceinline__ F32Consts f32c(const KickParams& kp) {
    F32Consts c;
    c.gamref = (float)kp.gamref;
    c.betaref = (float)kp.betaref;
    c.grbr = (float)kp.grbr;
    c.pref = (float)kp.pref;
    c.m = (float)kp.m_e_eV;
    c.m2 = c.m * c.m;
    return c;
}
// momenta (eV/c) and energy (eV) of one particle, FP32
__device__ __forceinline__ void mom32(float xq, float yq, float d, const F32Consts& c, float& px, float& py,
                                      float& pz, float& E) {
    const float gamma = c.gamref * (1.0f + c.betaref * d);
    const float beta = sqrtf(1.0f - 1.0f / (gamma * gamma));
    const float g = gamma * beta / c.grbr;
    const float pz2 = sqrtf(g * g - xq * xq - yq * yq);
    px = xq * c.pref;
    py = yq * c.pref;
    pz = pz2 * c.pref;
    E = gamma * c.m;
}

// ---------------------------------------------------------------------------
// frame: sum of momenta (+ FP64: lab coordinates stored for later stages)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(PT) k_frame64(const double* __restrict__ rp, KickParams kp,
                                                double* __restrict__ xp, double* __restrict__ part) {
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
}

__global__ void __launch_bounds__(PT) k_frame32(const double* __restrict__ rp, KickParams kp,
                                                double* __restrict__ part) {
    __shared__ double sm[3 * 32];
    const F32Consts c = f32c(kp);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const int64_t n = kp.n, ld = kp.ld;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float px, py, pz, E;
        mom32((float)rp[ld + i], (float)rp[3 * ld + i], (float)rp[5 * ld + i], c, px, py, pz, E);
        a0 += px;
        a1 += py;
        a2 += pz;
    }
    double acc[3] = {a0, a1, a2};
    block_sum<3>(acc, sm);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) part[blockIdx.x * 3 + k] = acc[k];
}

// one block: mean momentum -> basis T, gamma0, beta0 (sc.py:224-239, 243-248)
__global__ void k_frame_finalize(const double* __restrict__ part, int nblk, KickParams kp, ScState* st) {
    __shared__ double sm[3 * 32];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        for (int k = 0; k < 3; ++k) acc[k] += part[b * 3 + k];
    block_sum<3>(acc, sm);
    if (threadIdx.x != 0) return;
    const double nn = (double)kp.n;
    double t3[3] = {__ddiv_rn(acc[0], nn), __ddiv_rn(acc[1], nn), __ddiv_rn(acc[2], nn)};
    const double Pav = __dsqrt_rn(__fma_rn(t3[2], t3[2], __fma_rn(t3[1], t3[1], __dmul_rn(t3[0], t3[0]))));
    for (int k = 0; k < 3; ++k) t3[k] = __ddiv_rn(t3[k], Pav);
    // t1 = cross(ey, t3) = (t3z, 0, -t3x), normalised
    double t1[3] = {t3[2], 0.0, -t3[0]};
    const double n1 = __dsqrt_rn(__fma_rn(t1[2], t1[2], __fma_rn(t1[1], t1[1], __dmul_rn(t1[0], t1[0]))));
    for (int k = 0; k < 3; ++k) t1[k] = __ddiv_rn(t1[k], n1);
    // t2 = cross(t3, t1)
    const double t2[3] = {__dsub_rn(__dmul_rn(t3[1], t1[2]), __dmul_rn(t3[2], t1[1])),
                          __dsub_rn(__dmul_rn(t3[2], t1[0]), __dmul_rn(t3[0], t1[2])),
                          __dsub_rn(__dmul_rn(t3[0], t1[1]), __dmul_rn(t3[1], t1[0]))};
    for (int i = 0; i < 3; ++i) {
        st->T[i][0] = t1[i];
        st->T[i][1] = t2[i];
        st->T[i][2] = t3[i];
    }
    const double pm = __ddiv_rn(Pav, kp.m_e_eV);
    const double gamma0 = __dsqrt_rn(__dadd_rn(__dmul_rn(pm, pm), 1.0));
    const double beta0 = __dsqrt_rn(__dsub_rn(1.0, __drcp_rn(__dmul_rn(gamma0, gamma0))));
    st->Pav = Pav;
    st->gamma0 = gamma0;
    st->beta0 = beta0;
    st->kxy = __dmul_rn(kp.cdT, __dsub_rn(1.0, __dmul_rn(beta0, beta0)));
    st->kz = kp.cdT;
    int status = SC_OK;
    if (!(Pav > 0.0) || !isfinite(Pav) || !isfinite(gamma0) || !isfinite(t1[0]) || !isfinite(t2[1])) status = SC_ERR_NONFINITE;
    st->status = status;
}

// ---------------------------------------------------------------------------
// extent: rotated positions (z scaled by gamma0), min/max, charge moments
// part layout per block: min[3], max[3], sum q*x[3], sum q
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void extent_block_out(double (&mn)[3], double (&mx)[3], double (&qs)[4], double* sm,
                                                 double* part) {
    block_minmax<3, false>(mn, sm);
    block_minmax<3, true>(mx, sm);
    block_sum<4>(qs, sm);
    if (threadIdx.x == 0) {
        double* o = part + blockIdx.x * 10;
        for (int k = 0; k < 3; ++k) {
            o[k] = mn[k];
            o[3 + k] = mx[k];
            o[6 + k] = qs[k];
        }
        o[9] = qs[3];
    }
}

__global__ void __launch_bounds__(PT) k_extent64(const double* __restrict__ xp, const double* __restrict__ q,
                                                 KickParams kp, double* __restrict__ X, double* __restrict__ part,
                                                 const ScState* st) {
    __shared__ double sm[4 * 32];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    double qs[4] = {0.0, 0.0, 0.0, 0.0};
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
            X[j * n + i] = v[j];
            mn[j] = fmin(mn[j], v[j]);
            mx[j] = fmax(mx[j], v[j]);
            qs[j] += qi * v[j];
        }
        qs[3] += qi;
    }
    extent_block_out<double>(mn, mx, qs, sm, part);
}

__global__ void __launch_bounds__(PT) k_extent32(const double* __restrict__ rp, const double* __restrict__ q,
                                                 KickParams kp, float* __restrict__ X, double* __restrict__ part,
                                                 const ScState* st) {
    __shared__ double sm[4 * 32];
    const F32Consts c = f32c(kp);
    float mnf[3] = {INFINITY, INFINITY, INFINITY}, mxf[3] = {-INFINITY, -INFINITY, -INFINITY};
    float qsf[4] = {0.f, 0.f, 0.f, 0.f};
    const int64_t n = kp.n, ld = kp.ld;
    const bool ok = st->status == SC_OK;
    float T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = (float)st->T[i][j];
    const float g0 = (float)st->gamma0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ok && i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float xq = (float)rp[ld + i], yq = (float)rp[3 * ld + i], d = (float)rp[5 * ld + i];
        const float tau = (float)rp[4 * ld + i];
        float px, py, pz, E;
        mom32(xq, yq, d, c, px, py, pz, E);
        const float s = tau / E;
        const float l0 = (float)rp[i] - px * s, l1 = (float)rp[2 * ld + i] - py * s, l2 = -pz * s;
        float v[3];
        for (int j = 0; j < 3; ++j) v[j] = l0 * T[0][j] + l1 * T[1][j] + l2 * T[2][j];
        v[2] *= g0;
        const float qi = (float)q[i];
        for (int j = 0; j < 3; ++j) {
            X[j * n + i] = v[j];
            mnf[j] = fminf(mnf[j], v[j]);
            mxf[j] = fmaxf(mxf[j], v[j]);
            qsf[j] += qi * v[j];
        }
        qsf[3] += qi;
    }
    double mn[3] = {mnf[0], mnf[1], mnf[2]}, mx[3] = {mxf[0], mxf[1], mxf[2]};
    double qs[4] = {qsf[0], qsf[1], qsf[2], qsf[3]};
    extent_block_out<float>(mn, mx, qs, sm, part);
}

// el_field entry: X given as [n][3] rotated positions; z scaled by gamma in place
template <typename R>
__global__ void __launch_bounds__(PT) k_extent_xyz(double* __restrict__ Xin, const double* __restrict__ q, int64_t n,
                                                   double gamma, R* __restrict__ X, double* __restrict__ part) {
    __shared__ double sm[4 * 32];
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    double qs[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v[3] = {Xin[3 * i], Xin[3 * i + 1], __dmul_rn(Xin[3 * i + 2], gamma)};
        Xin[3 * i + 2] = v[2];
        const double qi = q[i];
        for (int j = 0; j < 3; ++j) {
            X[j * n + i] = (R)v[j];
            mn[j] = fmin(mn[j], v[j]);
            mx[j] = fmax(mx[j], v[j]);
            qs[j] += qi * v[j];
        }
        qs[3] += qi;
    }
    extent_block_out<R>(mn, mx, qs, sm, part);
}

// one block: steps, X_off, potential scale, Green cache check (sc.py:172-186, 167)
__global__ void k_mesh_finalize(const double* __restrict__ part, int nblk, KickParams kp, ScState* st,
                                double gamma_override) {
    __shared__ double sm[4 * 32];
    if (gamma_override > 0.0 && threadIdx.x == 0) st->status = SC_OK;
    __syncthreads();
    const bool ok = st->status == SC_OK;
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    double qs[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        const double* o = part + b * 10;
        for (int k = 0; k < 3; ++k) {
            mn[k] = fmin(mn[k], o[k]);
            mx[k] = fmax(mx[k], o[3 + k]);
            qs[k] += o[6 + k];
        }
        qs[3] += o[9];
    }
    block_minmax<3, false>(mn, sm);
    block_minmax<3, true>(mx, sm);
    block_sum<4>(qs, sm);
    if (threadIdx.x != 0 || !ok) return;
    if (gamma_override > 0.0) st->gamma0 = gamma_override;
    const int nm[3] = {kp.nx, kp.ny, kp.nz};
    double steps[3], xoff[3];
    bool bad = !(qs[3] != 0.0) || !isfinite(qs[3]);
    for (int k = 0; k < 3; ++k) {
        double XX = __dsub_rn(mx[k], mn[k]);
        if (!isnan(kp.mesh_scale)) XX = __dmul_rn(XX, kp.mesh_scale);
        steps[k] = __ddiv_rn(XX, (double)(nm[k] - 3));
        const double xmin = __ddiv_rn(mn[k], steps[k]);
        const double xmid = __ddiv_rn(__ddiv_rn(qs[k], steps[k]), qs[3]);
        xoff[k] = __dadd_rn(floor(__dsub_rn(xmin, xmid)), xmid);
        if (!isnan(kp.mesh_shift)) xoff[k] = __dadd_rn(xoff[k], kp.mesh_shift);
        if (!(steps[k] > 0.0) || !isfinite(steps[k]) || !isfinite(xoff[k])) bad = true;
    }
    if (bad) {
        st->status = SC_ERR_DEGENERATE;
        return;
    }
    for (int k = 0; k < 3; ++k) {
        st->steps[k] = steps[k];
        st->xoff[k] = xoff[k];
    }
    st->phi_denom = __dmul_rn(__dmul_rn(__dmul_rn(kp.four_pi_eps0, steps[0]), steps[1]), steps[2]);
    st->phi_norm = 1.0 / ((double)kp.Mx * (double)kp.My * (double)kp.Mz);
    const bool same = steps[0] == st->igf_h[0] && steps[1] == st->igf_h[1] && steps[2] == st->igf_h[2];
    st->igf_rebuild = same ? 0 : 1;
    for (int k = 0; k < 3; ++k) st->igf_h[k] = steps[k];
}

// potential entry: explicit spacing
__global__ void k_set_mesh(ScState* st, double hx, double hy, double hz, KickParams kp) {
    st->status = SC_OK;
    st->steps[0] = hx;
    st->steps[1] = hy;
    st->steps[2] = hz;
    st->phi_denom = __dmul_rn(__dmul_rn(__dmul_rn(kp.four_pi_eps0, hx), hy), hz);
    st->phi_norm = 1.0 / ((double)kp.Mx * (double)kp.My * (double)kp.Mz);
    const bool same = hx == st->igf_h[0] && hy == st->igf_h[1] && hz == st->igf_h[2];
    st->igf_rebuild = same ? 0 : 1;
    st->igf_h[0] = hx;
    st->igf_h[1] = hy;
    st->igf_h[2] = hz;
}

// ---------------------------------------------------------------------------
// keys: X = xyz/steps - X_off, key = (Xi*ny + Yi)*nz + Zi with Xi = floor(X)+1
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(PT) k_keys(R* __restrict__ X, uint32_t* __restrict__ keys, KickParams kp,
                                             ScState* st) {
    if (st->status) return;
    const int64_t n = kp.n;
    const double s0 = st->steps[0], s1 = st->steps[1], s2 = st->steps[2];
    const double o0 = st->xoff[0], o1 = st->xoff[1], o2 = st->xoff[2];
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R g[3];
        if (sizeof(R) == 8) {
            g[0] = (R)__dsub_rn(__ddiv_rn((double)X[i], s0), o0);
            g[1] = (R)__dsub_rn(__ddiv_rn((double)X[n + i], s1), o1);
            g[2] = (R)__dsub_rn(__ddiv_rn((double)X[2 * n + i], s2), o2);
        } else {
            g[0] = (R)((float)X[i] / (float)s0 - (float)o0);
            g[1] = (R)((float)X[n + i] / (float)s1 - (float)o1);
            g[2] = (R)((float)X[2 * n + i] / (float)s2 - (float)o2);
        }
        const R fx = floor(g[0]) + 1, fy = floor(g[1]) + 1, fz = floor(g[2]) + 1;
        const bool in = fx >= 0 && fy >= 0 && fz >= 0 && fx < kp.nx && fy < kp.ny && fz < kp.nz;
        uint32_t key = 0;
        if (in) key = ((uint32_t)fx * (uint32_t)kp.ny + (uint32_t)fy) * (uint32_t)kp.nz + (uint32_t)fz;
        else bad = true;
        keys[i] = key;
        X[i] = g[0];
        X[n + i] = g[1];
        X[2 * n + i] = g[2];
    }
    if (bad) atomicCAS(&st->status, SC_OK, SC_ERR_NONFINITE);
}

// ---------------------------------------------------------------------------
// trilinear gather, scipy.ndimage.map_coordinates(order=1, mode='constant')
// semantics: a sample outside [0, n-1] in any axis is 0
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R trilerp(const R* __restrict__ F, int nx, int ny, int nz, R c0, R c1, R c2) {
    if (!(c0 >= 0) || !(c1 >= 0) || !(c2 >= 0) || c0 > nx - 1 || c1 > ny - 1 || c2 > nz - 1) return 0;
    int i = (int)floor(c0), j = (int)floor(c1), k = (int)floor(c2);
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

__global__ void __launch_bounds__(PT) k_kick64(double* __restrict__ rp, const double* __restrict__ xp,
                                               const double* __restrict__ X, const double* __restrict__ ex,
                                               const double* __restrict__ ey, const double* __restrict__ ez,
                                               KickParams kp, const ScState* st) {
    if (st->status) return;
    const int64_t n = kp.n, ld = kp.ld;
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = st->T[i][j];
    const double g0 = st->gamma0, kxy = st->kxy, kz = st->kz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double e0, e1, e2;
        gather3<double>(ex, ey, ez, kp.nx, kp.ny, kp.nz, X[i], X[n + i], X[2 * n + i], e0, e1, e2);
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

__global__ void __launch_bounds__(PT) k_kick32(double* __restrict__ rp, const float* __restrict__ X,
                                               const float* __restrict__ ex, const float* __restrict__ ey,
                                               const float* __restrict__ ez, KickParams kp, const ScState* st) {
    if (st->status) return;
    const int64_t n = kp.n, ld = kp.ld;
    const F32Consts c = f32c(kp);
    float T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = (float)st->T[i][j];
    const float g0 = (float)st->gamma0, kxy = (float)st->kxy, kz = (float)st->kz;
    const float ipref = 1.0f / c.pref;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float e0, e1, e2;
        gather3<float>(ex, ey, ez, kp.nx, kp.ny, kp.nz, X[i], X[n + i], X[2 * n + i], e0, e1, e2);
        const float d0 = kxy * e0 * g0, d1 = kxy * e1 * g0, d2 = kz * e2;  // kick in the beam frame
        const float dpx = T[0][0] * d0 + T[0][1] * d1 + T[0][2] * d2;
        const float dpy = T[1][0] * d0 + T[1][1] * d1 + T[1][2] * d2;
        const float dpz = T[2][0] * d0 + T[2][1] * d1 + T[2][2] * d2;
        const double r1 = rp[ld + i], r3 = rp[3 * ld + i], r4 = rp[4 * ld + i], r5 = rp[5 * ld + i];
        float px, py, pz, E;
        mom32((float)r1, (float)r3, (float)r5, c, px, py, pz, E);
        const float pxn = px + dpx, pyn = py + dpy, pzn = pz + dpz;
        const float En = sqrtf(pxn * pxn + pyn * pyn + pzn * pzn + c.m2);
        const float dE = (2.0f * (px * dpx + py * dpy + pz * dpz) + (dpx * dpx + dpy * dpy + dpz * dpz)) / (E + En);
        const float tau = (float)r4;
        const float dtau = tau * (pz * dE - E * dpz) / (E * pzn);
        const float iEE = 1.0f / (E * En);
        const float dx = tau * (dpx * E - px * dE) * iEE + (pxn / En) * dtau;
        const float dy = tau * (dpy * E - py * dE) * iEE + (pyn / En) * dtau;
        rp[i] = rp[i] + (double)dx;
        rp[ld + i] = r1 + (double)(dpx * ipref);
        rp[2 * ld + i] = rp[2 * ld + i] + (double)dy;
        rp[3 * ld + i] = r3 + (double)(dpy * ipref);
        rp[4 * ld + i] = r4 + (double)dtau;
        rp[5 * ld + i] = r5 + (double)(dE * ipref);
    }
}

template <typename R>
__global__ void __launch_bounds__(PT) k_gather_xyz(const R* __restrict__ X, const R* __restrict__ ex,
                                                   const R* __restrict__ ey, const R* __restrict__ ez,
                                                   double* __restrict__ out, KickParams kp, const ScState* st) {
    if (st->status) return;
    const int64_t n = kp.n;
    const double g0 = st->gamma0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        R e0, e1, e2;
        gather3<R>(ex, ey, ez, kp.nx, kp.ny, kp.nz, X[i], X[n + i], X[2 * n + i], e0, e1, e2);
        out[3 * i] = __dmul_rn((double)e0, g0);
        out[3 * i + 1] = __dmul_rn((double)e1, g0);
        out[3 * i + 2] = (double)e2;
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int particle_blocks(const Plan& p, int64_t n) {
    int64_t b = (n + PT - 1) / PT;
    if (b > p.part_blocks) b = p.part_blocks;
    return (int)(b > 0 ? b : 1);
}

cudaError_t launch_frame(const Plan& p, const Layout& L, char* ws, const KickParams& kp, const double* rp,
                         cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part_frame);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        k_frame64<<<nb, PT, 0, s>>>(rp, kp, reinterpret_cast<double*>(ws + L.xp), part);
    else
        k_frame32<<<nb, PT, 0, s>>>(rp, kp, part);
    k_frame_finalize<<<1, PT, 0, s>>>(part, nb, kp, st);
    return cudaGetLastError();
}

cudaError_t launch_extent(const Plan& p, const Layout& L, char* ws, const KickParams& kp, const double* rp,
                          const double* q, cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part_ext);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        k_extent64<<<nb, PT, 0, s>>>(reinterpret_cast<const double*>(ws + L.xp), q, kp,
                                     reinterpret_cast<double*>(ws + L.X), part, st);
    else
        k_extent32<<<nb, PT, 0, s>>>(rp, q, kp, reinterpret_cast<float*>(ws + L.X), part, st);
    k_mesh_finalize<<<1, PT, 0, s>>>(part, nb, kp, st, -1.0);
    return cudaGetLastError();
}

cudaError_t launch_extent_xyz(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double* X,
                              const double* q, double gamma, cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part_ext);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        k_extent_xyz<double><<<nb, PT, 0, s>>>(X, q, kp.n, gamma, reinterpret_cast<double*>(ws + L.X), part);
    else
        k_extent_xyz<float><<<nb, PT, 0, s>>>(X, q, kp.n, gamma, reinterpret_cast<float*>(ws + L.X), part);
    k_mesh_finalize<<<1, PT, 0, s>>>(part, nb, kp, st, gamma);
    return cudaGetLastError();
}

cudaError_t launch_set_mesh(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double hx, double hy,
                            double hz, cudaStream_t s) {
    (void)p;
    k_set_mesh<<<1, 1, 0, s>>>(reinterpret_cast<ScState*>(ws + L.state), hx, hy, hz, kp);
    return cudaGetLastError();
}

cudaError_t launch_keys(const Plan& p, const Layout& L, char* ws, const KickParams& kp, cudaStream_t s) {
    ScState* st = reinterpret_cast<ScState*>(ws + L.state);
    const int nb = particle_blocks(p, kp.n);
    uint32_t* keys = reinterpret_cast<uint32_t*>(ws + L.keys);
    if (p.prec == SC_FP64)
        k_keys<double><<<nb, PT, 0, s>>>(reinterpret_cast<double*>(ws + L.X), keys, kp, st);
    else
        k_keys<float><<<nb, PT, 0, s>>>(reinterpret_cast<float*>(ws + L.X), keys, kp, st);
    return cudaGetLastError();
}

cudaError_t launch_gather_kick(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double* rp,
                               cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        k_kick64<<<nb, PT, 0, s>>>(rp, reinterpret_cast<const double*>(ws + L.xp),
                                   reinterpret_cast<const double*>(ws + L.X), reinterpret_cast<const double*>(ws + L.ex),
                                   reinterpret_cast<const double*>(ws + L.ey), reinterpret_cast<const double*>(ws + L.ez),
                                   kp, st);
    else
        k_kick32<<<nb, PT, 0, s>>>(rp, reinterpret_cast<const float*>(ws + L.X), reinterpret_cast<const float*>(ws + L.ex),
                                   reinterpret_cast<const float*>(ws + L.ey), reinterpret_cast<const float*>(ws + L.ez),
                                   kp, st);
    return cudaGetLastError();
}

cudaError_t launch_gather_xyz(const Plan& p, const Layout& L, char* ws, const KickParams& kp, double* exyz,
                              cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int nb = particle_blocks(p, kp.n);
    if (p.prec == SC_FP64)
        k_gather_xyz<double><<<nb, PT, 0, s>>>(reinterpret_cast<const double*>(ws + L.X),
                                               reinterpret_cast<const double*>(ws + L.ex),
                                               reinterpret_cast<const double*>(ws + L.ey),
                                               reinterpret_cast<const double*>(ws + L.ez), exyz, kp, st);
    else
        k_gather_xyz<float><<<nb, PT, 0, s>>>(reinterpret_cast<const float*>(ws + L.X),
                                              reinterpret_cast<const float*>(ws + L.ex),
                                              reinterpret_cast<const float*>(ws + L.ey),
                                              reinterpret_cast<const float*>(ws + L.ez), exyz, kp, st);
    return cudaGetLastError();
}

}  // namespace ocsc
