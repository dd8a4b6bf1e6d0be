// Integrated Green's function (IGF) table and its spectrum.
//
// k_igf_corners/k_igf_diff restate SpaceCharge.sym_kernel
// (ocelot/cpbd/sc.py:109-133): the antiderivative IG of 1/r is evaluated in
// FP64 on the (nx+1)(ny+1)(nz+1) cell corners (x = hx*i - hx/2, ...), with
// the same operation order as the reference, and the 8-corner difference
// gives the integral of 1/r over each cell of the lag octant.  The corners
// are evaluated once each; the difference cancels catastrophically far from
// the origin, which is why this stage stays FP64 in both precision forms.
//
// The spectrum of the mirrored kernel (sc.py:142-149) is real and even in
// each axis, so it is built as three passes of real-even transforms over the
// octant (S1 along z, S2 along y, S3 along x).  Two real-even lines are
// packed into the real and imaginary parts of one complex FFT; for even input
// the real part of the result is the first line's spectrum and the imaginary
// part the second's.  The output G[kx][ky][kz] covers kx <= Mx/2,
// ky <= My/2, kz <= Mz/2 and is looked up with |k| folding by the x pass of
// the convolution.
//
// All kernels here return immediately unless ScState::igf_rebuild is set
// (the mesh spacing changed since the table in the workspace was built) or
// the caller forces a build.
#include <mutex>

#include "sc_common.cuh"
#include "sc_fft_dev.cuh"

namespace ocsc {

struct IgfArgs {
    double hx, hy, hz;
    int use_state;  // take the spacing from ScState::steps
    int force;      // build even if the cache is valid
    int hybrid;     // FP32 form: 8-corner formula only inside the near box
};

__device__ __forceinline__ bool igf_skip(const ScState* st, const IgfArgs& a) {
    if (a.force) return false;
    return st->status != SC_OK || !st->igf_rebuild;
}

__device__ __forceinline__ void igf_spacing(const ScState* st, const IgfArgs& a, double& hx, double& hy, double& hz) {
    hx = a.hx; hy = a.hy; hz = a.hz;
    if (a.use_state) { hx = st->steps[0]; hy = st->steps[1]; hz = st->steps[2]; }
}

// Near box of the hybrid table (igf_box_of in sc_common.cuh): computed once
// per kick with the mesh step and kept in the state; the full octant when
// the table is exact.  Cells long along z take the transverse box of the
// line form (igf_tbox_of).
__device__ __forceinline__ void igf_box(const ScState* st, int nx, int ny, int nz, int hybrid, int b[3]) {
    if (!hybrid) { b[0] = nx; b[1] = ny; b[2] = nz; return; }
    const bool line = st->igf_line;
    b[0] = line ? st->igf_tbox[0] : st->igf_box[0];
    b[1] = line ? st->igf_tbox[1] : st->igf_box[1];
    b[2] = st->igf_box[2];
}

__device__ __forceinline__ double igf_point(double x, double y, double z) {
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    const double t1 = __dmul_rn(__dmul_rn(__dmul_rn(-x, x), 0.5), atan(__ddiv_rn(__dmul_rn(y, z), __dmul_rn(x, r))));
    const double t2 = __dmul_rn(__dmul_rn(y, z), log(__dadd_rn(x, r)));
    const double t3 = __dmul_rn(__dmul_rn(__dmul_rn(y, y), 0.5), atan(__ddiv_rn(__dmul_rn(z, x), __dmul_rn(y, r))));
    const double t4 = __dmul_rn(__dmul_rn(z, x), log(__dadd_rn(y, r)));
    const double t5 = __dmul_rn(__dmul_rn(__dmul_rn(z, z), 0.5), atan(__ddiv_rn(__dmul_rn(x, y), __dmul_rn(z, r))));
    const double t6 = __dmul_rn(__dmul_rn(x, y), log(__dadd_rn(z, r)));
    return __dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(t1, t2), t3), t4), t5), t6);
}

// Line form of the integral of 1/r over the cell centred at (X, Y, Z >= 0)
// with half-widths (a, b, c), for cells at least 5 max(2a, 2b) from the z
// axis: exact along z,
//   L(rho) = asinh((Z + c) / rho) - asinh((Z - c) / rho),
// and the 3 x 3 Gauss-Legendre product rule across the cell (the transverse
// integrand is smooth there: the rule's error is below 1e-10 relative).  L is
// formed without cancellation: for Z > c as log1p(r - 1) of the ratio
// r = (u + su) / (v + sv), u, v = (Z +- c) / rho, su, sv = sqrt(1 + u^2),
// sqrt(1 + v^2), with
//   r - 1 = (2c / rho) (1 + (u + v) / (su + sv)) / (v + sv);
// for Z <= c as asinh(u) + asinh(-v).  Every term is positive, so the FP32
// result is within a few roundings (2e-7 relative, checked against a
// 40-digit evaluation of the 8-corner formula) of the exact integral.
__device__ __forceinline__ float line_L(float r2, float Z, float c) {
    const float irho = 1.0f / sqrtf(r2);
    const float u = (Z + c) * irho, v = (Z - c) * irho;
    if (!(v > 0.0f)) return asinhf(u) + asinhf(-v);
    const float su = sqrtf(1.0f + u * u), sv = sqrtf(1.0f + v * v);
    return log1pf((2.0f * c * irho) * (1.0f + (u + v) / (su + sv)) / (v + sv));
}
__device__ __forceinline__ float cell_line(float X, float Y, float Z, float a, float b, float c) {
    const float t[3] = {-0.77459666924148337704f, 0.0f, 0.77459666924148337704f};  // +-sqrt(3/5), 0
    const float w[3] = {0.55555555555555555556f, 0.88888888888888888889f, 0.55555555555555555556f};
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float x = X + a * t[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float y = Y + b * t[j];
            s = s + (w[i] * w[j]) * line_L(x * x + y * y, Z, c);
        }
    }
    return a * b * s;
}

// One of the six terms of igf_point (term 0..5: t1..t6), with the same
// operations, so that their sum in igf_point's order is its result bit for
// bit.  Terms 0, 2, 4 take an arctangent, 1, 3, 5 a logarithm.
__device__ __forceinline__ double igf_term(double x, double y, double z, int term) {
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    switch (term) {
        case 0: return __dmul_rn(__dmul_rn(__dmul_rn(-x, x), 0.5), atan(__ddiv_rn(__dmul_rn(y, z), __dmul_rn(x, r))));
        case 1: return __dmul_rn(__dmul_rn(y, z), log(__dadd_rn(x, r)));
        case 2: return __dmul_rn(__dmul_rn(__dmul_rn(y, y), 0.5), atan(__ddiv_rn(__dmul_rn(z, x), __dmul_rn(y, r))));
        case 3: return __dmul_rn(__dmul_rn(z, x), log(__dadd_rn(y, r)));
        case 4: return __dmul_rn(__dmul_rn(__dmul_rn(z, z), 0.5), atan(__ddiv_rn(__dmul_rn(x, y), __dmul_rn(z, r))));
        default: return __dmul_rn(__dmul_rn(x, y), log(__dadd_rn(z, r)));
    }
}

// corner c of a box with corner strides (cy1 * cz1, cz1, 1): its coordinates
__device__ __forceinline__ void igf_corner_xyz(unsigned c, int cy1, int cz1, double hx, double hy, double hz,
                                               double& x, double& y, double& z) {
    const unsigned t = c / (unsigned)cz1;
    const int k = (int)(c - t * (unsigned)cz1);
    const int i = (int)(t / (unsigned)cy1);
    const int j = (int)(t - (unsigned)i * cy1);
    x = __dsub_rn(__dmul_rn(hx, (double)i), __dmul_rn(hx, 0.5));
    y = __dsub_rn(__dmul_rn(hy, (double)j), __dmul_rn(hy, 0.5));
    z = __dsub_rn(__dmul_rn(hz, (double)k), __dmul_rn(hz, 0.5));
}

constexpr int IGF_THREADS = 256;
constexpr int IGF_SPLIT = IGF_THREADS / 6;  // corners per block per round in the split form

// IG on the corners of the near box (the whole octant when not hybrid),
// stored with the box's corner strides.
// The whole octant (the exact table): one thread per corner, bound by the
// FP64 pipe.  The near box of the hybrid table has a few hundred corners, so
// the time is the latency of one igf_point -- on this GPU's narrow FP64 pipe
// some 20 us of dependent arithmetic through three arctangents and three
// logarithms.  There each corner's six terms go to six threads (the
// arctangents in one half of the block, the logarithms in the other, so no
// warp runs both) and a seventh sums them in igf_point's order through shared
// memory: the same bits in a third of the time.  For cells long along z the
// line-form cells of the table (k1) are computed by the other blocks of the
// same launch meanwhile; blocks [0, bc) take the corners.
template <typename R>
__device__ __forceinline__ void igf_corners_body(double* __restrict__ ig, R* __restrict__ k1, int nx, int ny, int nz,
                                                 const IgfArgs& a, const ScState* st, VBlk vb) {
    __shared__ double terms[6 * IGF_SPLIT];
    if (igf_skip(st, a)) return;
    double hx, hy, hz;
    igf_spacing(st, a, hx, hy, hz);
    int b[3];
    igf_box(st, nx, ny, nz, a.hybrid, b);
    const int cx1 = b[0] + 1, cy1 = b[1] + 1, cz1 = b[2] + 1;
    // 32-bit index arithmetic: a mesh has fewer than 2^31 corners
    const unsigned total = (unsigned)cx1 * cy1 * cz1;
    const long long all = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    if (!a.hybrid) {
        for (unsigned c = vb.x * blockDim.x + threadIdx.x; c < total; c += vb.nx * blockDim.x) {
            double x, y, z;
            igf_corner_xyz(c, cy1, cz1, hx, hy, hz, x, y, z);
            if (!SC_IDX_OK(st, 31, c, all)) continue;
            ig[c] = igf_point(x, y, z);
        }
        return;
    }
    const bool line = st->igf_line;
    const int nblk = vb.nx;
    int bc = nblk;  // blocks on the corners
    if (line && nblk > 1) {
        const int want = (int)((total + IGF_SPLIT - 1) / IGF_SPLIT);
        bc = want < nblk - 1 ? want : nblk - 1;
    }
    if (vb.x < bc) {
        // term m of corner e of the round: thread (m % 2) * 3 * IGF_SPLIT + (m / 2) * IGF_SPLIT + e
        const int tid = threadIdx.x;
        const int half = tid / (3 * IGF_SPLIT), rem = tid - half * 3 * IGF_SPLIT;
        const int m = 2 * (rem / IGF_SPLIT) + half, e = rem % IGF_SPLIT;  // m: 0,2,4 atan; 1,3,5 log
        for (unsigned c0 = vb.x * IGF_SPLIT; c0 < total; c0 += bc * IGF_SPLIT) {
            const unsigned c = c0 + e;
            if (tid < 6 * IGF_SPLIT && c < total) {
                double x, y, z;
                igf_corner_xyz(c, cy1, cz1, hx, hy, hz, x, y, z);
                terms[m * IGF_SPLIT + e] = igf_term(x, y, z, m);
            }
            __syncthreads();
            if (tid < IGF_SPLIT && c0 + tid < total && SC_IDX_OK(st, 31, c0 + tid, all)) {
                const double* t = terms + tid;
                ig[c0 + tid] = __dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(__dadd_rn(t[0], t[IGF_SPLIT]), t[2 * IGF_SPLIT]),
                                                             t[3 * IGF_SPLIT]),
                                                   t[4 * IGF_SPLIT]),
                                         t[5 * IGF_SPLIT]);
            }
            __syncthreads();
        }
    }
    if (line && (vb.x >= bc || nblk == 1)) {
        // the line-form cells: k below the near box, (i, j) outside it
        const float hxf = a.use_state ? st->stepsf[0] : (float)hx;
        const float hyf = a.use_state ? st->stepsf[1] : (float)hy;
        const float hzf = a.use_state ? st->stepsf[2] : (float)hz;
        const int lb = nblk == 1 ? 0 : vb.x - bc, nlb = nblk == 1 ? 1 : nblk - bc;
        const unsigned ncl = (unsigned)nx * ny * b[2];
        for (unsigned c = lb * blockDim.x + threadIdx.x; c < ncl; c += nlb * blockDim.x) {
            const unsigned t = c / (unsigned)b[2];
            const int k = (int)(c - t * (unsigned)b[2]);
            const int i = (int)(t / (unsigned)ny);
            const int j = (int)(t - (unsigned)i * ny);
            if (i < b[0] && j < b[1]) continue;
            const unsigned o = ((unsigned)i * ny + j) * nz + k;
            if (!SC_IDX_OK(st, 35, o, (long long)nx * ny * nz)) continue;
            k1[o] = (R)cell_line((float)i * hxf, (float)j * hyf, (float)k * hzf, 0.5f * hxf, 0.5f * hyf, 0.5f * hzf);
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(IGF_THREADS) k_igf_corners(double* __restrict__ ig, R* __restrict__ k1, int nx,
                                                             int ny, int nz, IgfArgs a, const ScState* st) {
    pdl_wait();
    igf_corners_body<R>(ig, k1, nx, ny, nz, a, st, hw_vblk());
}

// 4th-order multipole form of the integral of 1/r over the cell centred at
// (X,Y,Z) with half-widths (a,b,c), in FP32:
//   V/R [1 + (a^2(3x^2-1) + b^2(3y^2-1) + c^2(3z^2-1)) / (6 R^2)
//        + (sum a^4 F4(x^2)/120 + sum a^2 b^2 F22(x^2,y^2)/36) / R^4],
//   x = X/R, ..., F4(u) = 3(35u^2 - 30u + 3), F22(u,v) = 3(35uv - 5(u+v) + 1)
// (the Taylor expansion of 1/|R+s| averaged over the box; odd orders vanish)
__device__ __forceinline__ float cell_multipole(float X, float Y, float Z, float a2, float b2, float c2, float V) {
    const float R2 = X * X + Y * Y + Z * Z;
    const float iR2 = 1.0f / R2, iR = rsqrtf(R2);
    const float x2 = X * X * iR2, y2 = Y * Y * iR2, z2 = Z * Z * iR2;
    const float A = a2 * iR2, B = b2 * iR2, Cc = c2 * iR2;
    const float t2 = (A * (3.f * x2 - 1.f) + B * (3.f * y2 - 1.f) + Cc * (3.f * z2 - 1.f)) * (1.0f / 6.0f);
    const float f4x = 3.f * (35.f * x2 * x2 - 30.f * x2 + 3.f);
    const float f4y = 3.f * (35.f * y2 * y2 - 30.f * y2 + 3.f);
    const float f4z = 3.f * (35.f * z2 * z2 - 30.f * z2 + 3.f);
    const float fxy = 3.f * (35.f * x2 * y2 - 5.f * (x2 + y2) + 1.f);
    const float fxz = 3.f * (35.f * x2 * z2 - 5.f * (x2 + z2) + 1.f);
    const float fyz = 3.f * (35.f * y2 * z2 - 5.f * (y2 + z2) + 1.f);
    const float t4 = (A * A * f4x + B * B * f4y + Cc * Cc * f4z) * (1.0f / 120.0f) +
                     (A * B * fxy + A * Cc * fxz + B * Cc * fyz) * (1.0f / 36.0f);
    return V * iR * (1.0f + t2 + t4);
}

// cell integrals: the 8-corner difference of IG inside the near box (FP64),
// the multipole form outside it (FP32 form only; for cells long along z the
// corners kernel has written the line-form cells); written as R
template <typename R>
__device__ __forceinline__ void igf_diff_body(const double* __restrict__ ig, R* __restrict__ k1, int nx, int ny,
                                              int nz, const IgfArgs& a, const ScState* st, VBlk vb) {
    if (igf_skip(st, a)) return;
    double hx, hy, hz;
    igf_spacing(st, a, hx, hy, hz);
    int bx[3];
    igf_box(st, nx, ny, nz, a.hybrid, bx);
    // the FP32 spacing: the copies the mesh finalize stored (conversions
    // from FP64 issue on this GPU's slow FP64 pipe, so not once per thread)
    float hxf, hyf, hzf;
    if (a.use_state) {
        hxf = st->stepsf[0];
        hyf = st->stepsf[1];
        hzf = st->stepsf[2];
    } else {
        hxf = (float)hx;
        hyf = (float)hy;
        hzf = (float)hz;
    }
    const float a2 = 0.25f * hxf * hxf, b2 = 0.25f * hyf * hyf, c2 = 0.25f * hzf * hzf, V = hxf * hyf * hzf;
    const bool line = a.hybrid && st->igf_line;
    const unsigned total = (unsigned)nx * ny * nz;
    const unsigned sy = bx[2] + 1, sx = (unsigned)(bx[1] + 1) * (bx[2] + 1);
    for (unsigned c = vb.x * blockDim.x + threadIdx.x; c < total; c += vb.nx * blockDim.x) {
        const unsigned t = c / (unsigned)nz;
        const int k = (int)(c - t * (unsigned)nz);
        const int i = (int)(t / (unsigned)ny);
        const int j = (int)(t - (unsigned)i * ny);
        if (i < bx[0] && j < bx[1] && k < bx[2]) {
            const unsigned o = i * sx + j * sy + k;
            if (!SC_IDX_OK(st, 32, o + sx + sy + 1, (long long)(nx + 1) * (ny + 1) * (nz + 1))) continue;
            double v = __dsub_rn(ig[o + sx + sy + 1], ig[o + sy + 1]);
            v = __dsub_rn(v, ig[o + sx + 1]);
            v = __dadd_rn(v, ig[o + 1]);
            v = __dsub_rn(v, ig[o + sx + sy]);
            v = __dadd_rn(v, ig[o + sy]);
            v = __dadd_rn(v, ig[o + sx]);
            v = __dsub_rn(v, ig[o]);
            k1[c] = (R)v;
        } else if (line && k < bx[2]) {
            continue;  // the line form, written by the corners kernel
        } else {
            if (!SC_IDX_OK(st, 34, c, total)) continue;
            k1[c] = (R)cell_multipole((float)i * hxf, (float)j * hyf, (float)k * hzf, a2, b2, c2, V);
        }
    }
}

template <typename R>
__global__ void k_igf_diff(const double* __restrict__ ig, R* __restrict__ k1, int nx, int ny, int nz, IgfArgs a,
                           const ScState* st) {
    pdl_wait();
    igf_diff_body<R>(ig, k1, nx, ny, nz, a, st, hw_vblk());
}

// index of the even extension of a length-n octant to a period M (-1: zero)
__device__ __forceinline__ int even_src(int z, int n, int M) {
    if (z < n) return z;
    const int m = M - z;
    return m < n ? m : -1;
}

constexpr int GT = 256;
// complex lines (= 2 columns each) per block in the strided passes; fewer
// when two line buffers would not fit in shared memory (FP64 at M = 512)
template <typename R>
static inline int green_cols(int M) {
    int tk = 16;
    while (tk > 2 && sizeof(Cx<R>) * (size_t)(M + 2 * tk * fft_ls(M)) > 200 * 1024) tk /= 2;
    return tk;
}

// S1: along z; rows (x, y) of K1 -> S1[x][y][kz], kz <= Mz/2
template <typename R>
__device__ __forceinline__ void green_z_body(const R* __restrict__ k1, R* __restrict__ s1, int ny, int nz, int Kz,
                                             const RadixPlan& rz, const Cx<R>* __restrict__ twg, int NC,
                                             const IgfArgs& a, const ScState* st, VBlk vb) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (igf_skip(st, a)) return;
    const int Mz = rz.L, lz = fft_ls(Mz);
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* A = tw + Mz;
    Cx<R>* B = A + NC * lz;
    load_twiddles<R>(tw, twg, Mz);
    const int x = vb.y, y0 = vb.x * 2 * NC;
    constexpr int U = 4;  // elements per thread per round, their loads issued together
    for (DivWalk w(threadIdx.x, blockDim.x, Mz); w.q < NC;) {
        int cs[U], zz[U];
        R re[U], im[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            cs[u] = w.q;
            zz[u] = w.r;
            w.next();
            const int ya = y0 + 2 * cs[u], yb = ya + 1;
            const int zs = cs[u] < NC ? even_src(zz[u], nz, Mz) : -1;
            const bool ok = zs >= 0 && SC_IDX_OK(st, 33, ((long long)x * ny + (ya < ny ? ya : 0)) * nz + zs,
                                                 (long long)vb.ny * ny * nz);
            re[u] = (ok && ya < ny) ? k1[((size_t)x * ny + ya) * nz + zs] : (R)0;
            im[u] = (ok && yb < ny) ? k1[((size_t)x * ny + yb) * nz + zs] : (R)0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (cs[u] < NC) A[cs[u] * lz + zz[u]] = cx<R>(re[u], im[u]);
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, false>(A, B, lz, NC, rz, tw);
    for (DivWalk w(threadIdx.x, blockDim.x, Kz); w.q < NC; w.next()) {
        const int c = w.q, k = w.r;
        const int ya = y0 + 2 * c, yb = ya + 1;
        const Cx<R> v = res[c * lz + k];
        if (!SC_IDX_OK(st, 35, ((long long)x * ny + (yb < ny ? yb : ya)) * Kz + k, (long long)vb.ny * ny * Kz)) continue;
        if (ya < ny) s1[((size_t)x * ny + ya) * Kz + k] = v.x;
        if (yb < ny) s1[((size_t)x * ny + yb) * Kz + k] = v.y;
    }
}

template <typename R>
__global__ void __launch_bounds__(GT) k_green_z(const R* __restrict__ k1, R* __restrict__ s1, int ny, int nz,
                                                int Kz, RadixPlan rz, const Cx<R>* __restrict__ twg, int NC,
                                                IgfArgs a, const ScState* st) {
    pdl_wait();
    green_z_body<R>(k1, s1, ny, nz, Kz, rz, twg, NC, a, st, hw_vblk());
}

// S2/S3: strided passes over columns kz (paired), line axis of length n -> M,
// input rows in[(o*nin + l)*Kz + kz], output rows out[(o*nout + kl)*Kz + kz].
// The complex lines are the column pairs (2 pr, 2 pr + 1) of every outer index
// o < nouter, flattened as o * P + pr (P = ceil(Kz / 2)); block vb.x takes GTK
// consecutive ones, thread t the line t mod GTK (GTK a power of two).
template <typename R>
__device__ __forceinline__ void green_strided_body(const R* __restrict__ in, R* __restrict__ out, int n,
                                                   int nin_stride, int nout, int Kz, int outer_in_stride,
                                                   int outer_out_stride, int nouter, const RadixPlan& rp,
                                                   const Cx<R>* __restrict__ twg, int GTK, const IgfArgs& a,
                                                   const ScState* st, VBlk vb) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (igf_skip(st, a)) return;
    const int M = rp.L, ls = fft_ls(M);
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* A = tw + M;
    Cx<R>* B = A + GTK * ls;
    load_twiddles<R>(tw, twg, M);
    const ColMap cm(GTK);
    const int P = (Kz + 1) / 2;
    const int f = vb.x * GTK + cm.kk;
    const bool live = f < nouter * P;
    const int o = f / P, pr = f - o * P;
    const int ka = 2 * pr, kb = ka + 1;
    const R* src = in + (size_t)o * outer_in_stride;
    R* dst = out + (size_t)o * outer_out_stride;
    Cx<R>* la = A + cm.kk * ls;
    constexpr int U = 8;  // rows per round: their loads are issued together
    for (int l0 = cm.r0; l0 < M; l0 += U * cm.rs) {
        R re[U], im[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int l = l0 + u * cm.rs;
            const int lsrc = (live && l < M) ? even_src(l, n, M) : -1;
            re[u] = (lsrc >= 0 && ka < Kz) ? src[(size_t)lsrc * nin_stride + ka] : (R)0;
            im[u] = (lsrc >= 0 && kb < Kz) ? src[(size_t)lsrc * nin_stride + kb] : (R)0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (l0 + u * cm.rs < M) la[l0 + u * cm.rs] = cx<R>(re[u], im[u]);
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, false>(A, B, ls, GTK, rp, tw);
    if (live)
        for (int l = cm.r0; l < nout; l += cm.rs) {
            const Cx<R> v = res[cm.kk * ls + l];
            if (ka < Kz) dst[(size_t)l * nin_stride + ka] = v.x;
            if (kb < Kz) dst[(size_t)l * nin_stride + kb] = v.y;
        }
}

template <typename R>
__global__ void __launch_bounds__(GT) k_green_strided(const R* __restrict__ in, R* __restrict__ out, int n,
                                                      int nin_stride, int nout, int Kz, int outer_in_stride,
                                                      int outer_out_stride, int nouter, RadixPlan rp,
                                                      const Cx<R>* __restrict__ twg, int GTK, IgfArgs a,
                                                      const ScState* st) {
    pdl_wait();
    green_strided_body<R>(in, out, n, nin_stride, nout, Kz, outer_in_stride, outer_out_stride, nouter, rp, twg, GTK,
                          a, st, hw_vblk());
}


static int grid_for(size_t work, int sm) {
    size_t b = (work + 255) / 256;
    size_t cap = (size_t)sm * 16;
    return (int)(b < cap ? (b ? b : 1) : cap);
}

cudaError_t launch_igf_h(const Plan& p, const Layout& L, char* ws, double* kern_out, double hx, double hy,
                         double hz, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    IgfArgs a;
    a.hx = hx; a.hy = hy; a.hz = hz;
    a.use_state = 0;
    a.force = 1;
    a.hybrid = 0;
    double* ig = reinterpret_cast<double*>(ws + L.igf_ig);
    const size_t nc = (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
    launch(k_igf_corners<double>, grid_for(nc, p.sm_count), IGF_THREADS, 0, s, ig, (double*)nullptr, p.nx, p.ny,
           p.nz, a, st);
    const size_t nk = (size_t)p.nx * p.ny * p.nz;
    launch(k_igf_diff<double>, grid_for(nk, p.sm_count), 256, 0, s, ig, kern_out, p.nx, p.ny, p.nz, a, st);
    return cudaGetLastError();
}

cudaError_t launch_igf(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    IgfArgs a;
    a.hx = a.hy = a.hz = 0;
    a.use_state = 1;
    a.force = 0;
    a.hybrid = p.exact_igf ? 0 : 1;
    double* ig = reinterpret_cast<double*>(ws + L.igf_ig);
    const size_t nc = (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
    // one block per SM: eight warps keep an SM's FP64 pipe busy, and the
    // registers left over hold the blocks of the concurrent particle kernels
    size_t gb = (nc + 255) / 256;
    if (gb > (size_t)p.sm_count) gb = (size_t)p.sm_count;
    const size_t nk = (size_t)p.nx * p.ny * p.nz;
    if (p.prec == SC_FP64)
        launch(k_igf_corners<double>, (int)gb, IGF_THREADS, 0, s, ig, reinterpret_cast<double*>(ws + L.igf_k1), p.nx,
               p.ny, p.nz, a, st);
    else
        launch(k_igf_corners<float>, (int)gb, IGF_THREADS, 0, s, ig, reinterpret_cast<float*>(ws + L.igf_k1), p.nx,
               p.ny, p.nz, a, st);
    if (p.prec == SC_FP64)
        launch(k_igf_diff<double>, grid_for(nk, p.sm_count), 256, 0, s, ig, reinterpret_cast<double*>(ws + L.igf_k1), p.nx,
                                                                     p.ny, p.nz, a, st);
    else
        launch(k_igf_diff<float>, grid_for(nk, p.sm_count), 256, 0, s, ig, reinterpret_cast<float*>(ws + L.igf_k1), p.nx,
                                                                    p.ny, p.nz, a, st);
    return cudaGetLastError();
}

template <typename R>
static cudaError_t spectrum_t(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    IgfArgs a;
    a.hx = a.hy = a.hz = 0;
    a.use_state = 1;
    a.force = 0;
    a.hybrid = 0;
    const int Kx = p.Mx / 2 + 1, Ky = p.My / 2 + 1, Kz = p.Mz / 2 + 1;
    const R* k1 = reinterpret_cast<const R*>(ws + L.igf_k1);
    R* s1 = reinterpret_cast<R*>(ws + L.green_s1);
    R* s2 = reinterpret_cast<R*>(ws + L.green_s2);
    R* g = reinterpret_cast<R*>(ws + L.green);
    const Cx<R>* twx = reinterpret_cast<const Cx<R>*>(ws + L.tw_x);
    const Cx<R>* twy = reinterpret_cast<const Cx<R>*>(ws + L.tw_y);
    const Cx<R>* twz = reinterpret_cast<const Cx<R>*>(ws + L.tw_z);
    cudaError_t e;
    int NC = 2048 / p.Mz;
    NC = NC < 1 ? 1 : (NC > 16 ? 16 : NC);
    const size_t smz = sizeof(Cx<R>) * (size_t)(p.Mz + 2 * NC * fft_ls(p.Mz));
    if ((e = set_smem(k_green_z<R>, smz))) return e;
    dim3 gz((p.ny + 2 * NC - 1) / (2 * NC), p.nx);
    launch(k_green_z<R>, gz, GT, smz, s, k1, s1, p.ny, p.nz, Kz, p.rz, twz, NC, a, st);
    // S2 along y: for each x, rows y < ny of S1[x] -> rows ky < Ky of S2[x]
    const int tky = green_cols<R>(p.My), tkx = green_cols<R>(p.Mx);
    const size_t smy = sizeof(Cx<R>) * (size_t)(p.My + 2 * tky * fft_ls(p.My));
    const size_t smx = sizeof(Cx<R>) * (size_t)(p.Mx + 2 * tkx * fft_ls(p.Mx));
    if ((e = set_smem(k_green_strided<R>, smx > smy ? smx : smy))) return e;
    const int P = (Kz + 1) / 2;  // column pairs per outer index
    dim3 gy((p.nx * P + tky - 1) / tky);
    launch(k_green_strided<R>, gy, GT, smy, s, s1, s2, p.ny, Kz, Ky, Kz, p.ny * Kz, Ky * Kz, p.nx, p.ry, twy, tky, a,
           st);
    // S3 along x: for each ky, rows x < nx of S2[.][ky] -> rows kx < Kx of G[.][ky]
    dim3 gx((Ky * P + tkx - 1) / tkx);
    launch(k_green_strided<R>, gx, GT, smx, s, s2, g, p.nx, Ky * Kz, Kx, Kz, Kz, Kz, Ky, p.rx, twx, tkx, a, st);
    return cudaGetLastError();
}

template <typename R>
static cudaError_t prepare_green_t(const Plan& p) {
    cudaError_t e;
    int NC = 2048 / p.Mz;
    NC = NC < 1 ? 1 : (NC > 16 ? 16 : NC);
    const size_t smz = sizeof(Cx<R>) * (size_t)(p.Mz + 2 * NC * fft_ls(p.Mz));
    const int tky = green_cols<R>(p.My), tkx = green_cols<R>(p.Mx);
    const size_t smy = sizeof(Cx<R>) * (size_t)(p.My + 2 * tky * fft_ls(p.My));
    const size_t smx = sizeof(Cx<R>) * (size_t)(p.Mx + 2 * tkx * fft_ls(p.Mx));
    if ((e = set_smem(k_green_z<R>, smz))) return e;
    return set_smem(k_green_strided<R>, smx > smy ? smx : smy);
}

cudaError_t prepare_green_kernels(const Plan& p) {
    return p.prec == SC_FP64 ? prepare_green_t<double>(p) : prepare_green_t<float>(p);
}

cudaError_t launch_green_spectrum(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    return p.prec == SC_FP64 ? spectrum_t<double>(p, L, ws, s) : spectrum_t<float>(p, L, ws, s);
}

// ---------------------------------------------------------------------------
// batched IGF table and spectrum (FP32 form): one launch per pass over every
// beam of a batch; each beam decides on the device whether its table needs a
// rebuild, as in the plain launches
// ---------------------------------------------------------------------------
#define BATCH_BEAM(stage)                                                       \
    const int b = batch_beam(start, nb);                                        \
    const BatchBeam& B = beams[b];                                              \
    const VBlk vb = batch_vblk(start, b, B.gx[stage], B.gy[stage]);             \
    char* ws = B.ws;                                                            \
    const Layout& L = B.L;                                                      \
    const Plan& p = B.p;                                                        \
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);

__device__ __forceinline__ IgfArgs batch_igf_args(const Plan& p, int hybrid_allowed) {
    IgfArgs a;
    a.hx = a.hy = a.hz = 0;
    a.use_state = 1;
    a.force = 0;
    a.hybrid = (hybrid_allowed && !p.exact_igf) ? 1 : 0;
    return a;
}

__global__ void __launch_bounds__(256) kb_igf_corners(const BatchBeam* __restrict__ beams,
                                                      const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_IGF_C)
    igf_corners_body<float>(reinterpret_cast<double*>(ws + L.igf_ig), reinterpret_cast<float*>(ws + L.igf_k1), p.nx,
                            p.ny, p.nz, batch_igf_args(p, 1), st, vb);
}

__global__ void __launch_bounds__(256) kb_igf_diff(const BatchBeam* __restrict__ beams,
                                                   const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_IGF_D)
    igf_diff_body<float>(reinterpret_cast<const double*>(ws + L.igf_ig), reinterpret_cast<float*>(ws + L.igf_k1),
                         p.nx, p.ny, p.nz, batch_igf_args(p, 1), st, vb);
}

__global__ void __launch_bounds__(GT) kb_green_z(const BatchBeam* __restrict__ beams, const int* __restrict__ start,
                                                 int nb) {
    pdl_wait();
    BATCH_BEAM(BS_GREEN_Z)
    green_z_body<float>(reinterpret_cast<const float*>(ws + L.igf_k1), reinterpret_cast<float*>(ws + L.green_s1),
                        p.ny, p.nz, p.Mz / 2 + 1, p.rz, reinterpret_cast<const Cx<float>*>(ws + L.tw_z), B.green_nc,
                        batch_igf_args(p, 0), st, vb);
}

// AXIS 1: S2 along y (S1 -> S2); AXIS 0: S3 along x (S2 -> G)
template <int AXIS>
__global__ void __launch_bounds__(GT) kb_green_strided(const BatchBeam* __restrict__ beams,
                                                       const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(AXIS == 1 ? BS_GREEN_Y : BS_GREEN_X)
    const int Kx = p.Mx / 2 + 1, Ky = p.My / 2 + 1, Kz = p.Mz / 2 + 1;
    if (AXIS == 1)
        green_strided_body<float>(reinterpret_cast<const float*>(ws + L.green_s1),
                                  reinterpret_cast<float*>(ws + L.green_s2), p.ny, Kz, Ky, Kz, p.ny * Kz, Ky * Kz,
                                  p.nx, p.ry, reinterpret_cast<const Cx<float>*>(ws + L.tw_y), B.green_tky,
                                  batch_igf_args(p, 0), st, vb);
    else
        green_strided_body<float>(reinterpret_cast<const float*>(ws + L.green_s2),
                                  reinterpret_cast<float*>(ws + L.green), p.nx, Ky * Kz, Kx, Kz, Kz, Kz, Ky, p.rx,
                                  reinterpret_cast<const Cx<float>*>(ws + L.tw_x), B.green_tkx, batch_igf_args(p, 0),
                                  st, vb);
}
#undef BATCH_BEAM

int batch_igf_blocks(const Plan& p, int diff) {
    const size_t work = diff ? (size_t)p.nx * p.ny * p.nz : (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
    const size_t cap = diff ? 64 : 32;
    size_t b = (work + 255) / 256;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

void batch_green_tiling(BatchBeam& B, size_t smem[3]) {
    const Plan& p = B.p;
    const int Ky = p.My / 2 + 1, Kz = p.Mz / 2 + 1;
    int NC = 2048 / p.Mz;
    B.green_nc = NC < 1 ? 1 : (NC > 16 ? 16 : NC);
    B.green_tky = green_cols<float>(p.My);
    B.green_tkx = green_cols<float>(p.Mx);
    B.gx[BS_IGF_C] = batch_igf_blocks(p, 0);
    B.gy[BS_IGF_C] = 1;
    B.gx[BS_IGF_D] = batch_igf_blocks(p, 1);
    B.gy[BS_IGF_D] = 1;
    B.gx[BS_GREEN_Z] = (p.ny + 2 * B.green_nc - 1) / (2 * B.green_nc);
    B.gy[BS_GREEN_Z] = p.nx;
    const int P = (Kz + 1) / 2;  // column pairs per outer index
    B.gx[BS_GREEN_Y] = (p.nx * P + B.green_tky - 1) / B.green_tky;
    B.gy[BS_GREEN_Y] = 1;
    B.gx[BS_GREEN_X] = (Ky * P + B.green_tkx - 1) / B.green_tkx;
    B.gy[BS_GREEN_X] = 1;
    smem[0] = sizeof(Cx<float>) * (size_t)(p.Mz + 2 * B.green_nc * fft_ls(p.Mz));
    smem[1] = sizeof(Cx<float>) * (size_t)(p.My + 2 * B.green_tky * fft_ls(p.My));
    smem[2] = sizeof(Cx<float>) * (size_t)(p.Mx + 2 * B.green_tkx * fft_ls(p.Mx));
}

cudaError_t prepare_batch_green() {
    cudaError_t e;
    const size_t big = 48 * 1024 + 1;
    if ((e = smem_opt_in(reinterpret_cast<const void*>(kb_green_z), big))) return e;
    if ((e = smem_opt_in(reinterpret_cast<const void*>(kb_green_strided<1>), big))) return e;
    return smem_opt_in(reinterpret_cast<const void*>(kb_green_strided<0>), big);
}

cudaError_t launch_batch_igf(const BatchBeam* beams, const int* start_c, const int* start_d, int nb, int blocks_c,
                             int blocks_d, cudaStream_t s) {
    if (nb <= 0) return cudaSuccess;
    launch(kb_igf_corners, blocks_c, 256, 0, s, beams, start_c, nb);
    launch(kb_igf_diff, blocks_d, 256, 0, s, beams, start_d, nb);
    return cudaGetLastError();
}

cudaError_t launch_batch_green(const BatchBeam* beams, const int* sz, const int* sy, const int* sx, int nb,
                               const int blocks[3], const size_t smem[3], cudaStream_t s) {
    if (nb <= 0) return cudaSuccess;
    launch(kb_green_z, blocks[0], GT, smem[0], s, beams, sz, nb);
    launch(kb_green_strided<1>, blocks[1], GT, smem[1], s, beams, sy, nb);
    launch(kb_green_strided<0>, blocks[2], GT, smem[2], s, beams, sx, nb);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Workspace-free IGF table (sc_sym_kernel_static)
//
// Some callers cannot allocate device memory at the point where they need the
// table: a process whose device memory is reserved up front by another
// allocator (a framework's memory pool, an online control application with a
// fixed memory budget), or code on a latency-critical path that must not call
// cudaMalloc/cudaFree, which can synchronise the device.  For them the corner
// table lives in one file-scope device array, allocated by the driver when
// the library's module is loaded and kept by every GPU that loads the
// library until the process exits.  The first kScratchState bytes of it hold
// a zeroed stand-in for the workspace state that the kernels are handed.
// ---------------------------------------------------------------------------
constexpr long long kStaticMaxCorners = SC_SYM_KERNEL_STATIC_MAX_CORNERS;
constexpr long long kScratchState = 64;  // doubles (512 bytes >= sizeof(ScState))
static __device__ __align__(256) double g_igf_scratch[kScratchState + kStaticMaxCorners];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_ptr[kMaxDevices] = {};  // device address of g_igf_scratch, per device
int g_scratch_sms[kMaxDevices] = {};
}  // namespace

// Once per device, with that device current: the device address of the
// scratch array (host code may not use the symbol itself as a pointer) and
// the SM count for the launch shape.
static cudaError_t static_scratch(int dev, double** ptr, int* sms) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_igf_scratch);
        if (e != cudaSuccess) return e;
        int sm = 0;
        e = cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        g_scratch_sms[dev] = sm;
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *ptr = g_scratch_ptr[dev];
    *sms = g_scratch_sms[dev];
    return cudaSuccess;
}

}  // namespace ocsc

extern "C" int sc_sym_kernel_static(int nx, int ny, int nz, double hx, double hy, double hz, double* kern,
                                    void* stream) {
    using namespace ocsc;
    if (nx < 1 || ny < 1 || nz < 1) return sc_report(SC_ERR_ARG, "sc_sym_kernel_static: mesh dimensions must be >= 1");
    const long long corners = ((long long)nx + 1) * ((long long)ny + 1) * ((long long)nz + 1);
    if (corners > kStaticMaxCorners)
        return sc_report(SC_ERR_UNSUPPORTED,
                         "sc_sym_kernel_static: (nx+1)(ny+1)(nz+1) = %lld corners exceeds the static table of %lld "
                         "(use sc_sym_kernel with a workspace for this mesh)",
                         corners, kStaticMaxCorners);
    if (!kern) return sc_report(SC_ERR_ARG, "sc_sym_kernel_static: kern is NULL");
    if (!(hx > 0 && hy > 0 && hz > 0) || !isfinite(hx * hy * hz))
        return sc_report(SC_ERR_ARG, "sc_sym_kernel_static: mesh steps must be > 0");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sc_report(SC_ERR_CUDA, "sc_sym_kernel_static: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return sc_report(SC_ERR_UNSUPPORTED, "sc_sym_kernel_static: device %d", dev);
    double* base = nullptr;
    int sms = 0;
    e = static_scratch(dev, &base, &sms);
    if (e != cudaSuccess)
        return sc_report(SC_ERR_CUDA, "sc_sym_kernel_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    cudaStream_t s = (cudaStream_t)stream;
    ScState* st = reinterpret_cast<ScState*>(base);
    double* ig = base + kScratchState;
    // the state stand-in starts at zero (only its check fields are ever written)
    e = cudaMemsetAsync(st, 0, sizeof(ScState), s);
    if (e != cudaSuccess) return sc_report(SC_ERR_CUDA, "sc_sym_kernel_static: %s", cudaGetErrorString(e));
    IgfArgs a;
    a.hx = hx; a.hy = hy; a.hz = hz;
    a.use_state = 0;
    a.force = 1;
    a.hybrid = 0;
    launch(k_igf_corners<double>, grid_for((size_t)corners, sms), IGF_THREADS, 0, s, ig, (double*)nullptr, nx, ny, nz,
           a, st);
    launch(k_igf_diff<double>, grid_for((size_t)nx * ny * nz, sms), 256, 0, s, ig, kern, nx, ny, nz, a, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return sc_report(SC_ERR_CUDA, "sc_sym_kernel_static: %s", cudaGetErrorString(e));
    return SC_OK;
}
