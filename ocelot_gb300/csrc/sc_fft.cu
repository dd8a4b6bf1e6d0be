// Free-space potential by zero-padded FFT convolution with the integrated
// Green's function, and the forward-difference field grids.
//
// Restates SpaceCharge.potential (ocelot/cpbd/sc.py:135-168) and the field
// grids of el_field (sc.py:195-200).  The reference convolves on a
// (2N-1)^3 complex grid; the linear convolution is the same on any padded
// length M >= 2N-1, so each axis is padded to a length with a 2/4/8 radix
// plan.  Only the N^3 octant of the charge is non-zero and only the N^3
// octant of the result is kept, so the passes skip the zero planes:
//
//   F1  z: real-to-complex of the nx*ny charge lines (two lines per complex FFT)
//   F2  y: forward FFT of the nx*Kz columns, zero-padded from ny to My
//   F3  x: forward FFT, multiply by the real Green spectrum, inverse FFT,
//          keep x < nx (the only pass that sees all Mx planes, in shared memory)
//   B2  y: inverse FFT, keep y < ny
//   B1  z: complex-to-real of the nx*ny lines, keep z < nz, scale by
//          1/(Mx*My*Mz) and 1/(4*pi*eps0*hx*hy*hz)
//
// The complex work grid W[x][y][kz] (x < nx, y < My, kz <= Mz/2) stays in
// HBM/L2 between passes; each pass stages whole lines in shared memory.
#include "sc_common.cuh"
#include "sc_fft_dev.cuh"

namespace ocsc {

constexpr int FFT_THREADS = 256;

// complex lines (two real lines each) per block of the z passes: up to 8,
// so that a 64^3 mesh gives 256 blocks
static inline int z_lines_per_block(int Mz) {
    int nc = 1024 / Mz;
    return nc < 1 ? 1 : (nc > 8 ? 8 : nc);
}
// columns per block in the strided passes: 16, fewer when two line buffers
// of 16 columns would not fit in shared memory (FP64 at M = 512)
template <typename R>
static inline int strided_cols(int M, int nbuf = 2) {
    int tk = 16;
    while (tk > 2 && sizeof(Cx<R>) * (size_t)(M + nbuf * tk * fft_ls(M)) > 200 * 1024) tk /= 2;
    return tk;
}
// the plan's columns per block (SC_PARAM_FFT_COLS_X / _Y; 0: strided_cols),
// never more than fit.  The columns are independent lines, so the grouping
// changes no result.
template <typename R>
static inline int pass_cols(int want, int M, int nbuf = 2) {
    const int fit = strided_cols<R>(M, nbuf);
    return (want > 0 && want < fit) ? want : fit;
}

// Spectral fields (FP32 with SC_FP32_SPECTRAL_FIELDS).  The field grids are
// forward differences of the potential, Ex[i] = (phi[i] - phi[i+1]) / hx
// (sc.py:195-200); on the padded grid that difference is the product of the
// spectrum with D(k) = 1 - exp(2 pi i k / M), exact for every cell the
// reference keeps.  Taking it in Fourier space before the inverse transforms
// makes the rounding of each field relative to the field itself instead of
// to the potential, which is hundreds of times larger than the differences
// of neighbouring cells.
//   Ex: x inverse of (spectrum x D(kx)) into W2, then y and z inverses
//   Ey: y inverse of (W x D(ky)) into W3 (W after the x inverse), then z
//   Ez: z inverse of (y-inverted W) x D(kz)
// The potential itself is kept (z inverse of the y-inverted W).
template <typename R>
struct Spec {
    Cx<R>* W2;                       // the x-differenced grid (Ex); nullptr: no spectral fields
    Cx<R>* W3;                       // the y-differenced grid (Ey), separate passes only
    const Cx<R>* dx;                 // D(k) per axis
    const Cx<R>* dy;
    const Cx<R>* dz;
    R* ex;                           // field grids [nx][ny][nz], zero on their last plane
    R* ey;
    R* ez;
    int f0;                          // first output of the inverse passes: 0 with the potential, 1 without
};
template <typename R>
__device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
    return cx<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Stage the charge of NC complex z lines into the line buffer a (line c at
// a + c * lz): the real part of line c is row y0 + 2c of plane x, the
// imaginary part row y0 + 2c + 1, zero-padded from nz to Mz.  With qfix the
// charge arrives as the 64-bit fixed-point grid, is scaled to R and is also
// stored in q.  U elements per thread per round: all their loads are issued
// before any of them is converted or stored, one memory round trip per round.
// code, code + 1: the index-check codes of the two rows
template <typename R>
__device__ __forceinline__ void stage_charge_lines(R* __restrict__ q, const long long* __restrict__ qfix,
                                                   Cx<R>* __restrict__ a, int lz, int x, int y0, int NC, int ny,
                                                   int nz, int Mz, const ScState* st, long long ncell, int code) {
    constexpr int U = 4;
    const float ufix = qfix ? st->qfix_inv : 0.f;
    for (DivWalk w(threadIdx.x, blockDim.x, Mz); w.q < NC;) {
        int cs[U], zs[U];
        bool oka[U], okb[U];
        size_t ia[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            cs[u] = w.q;
            zs[u] = w.r;
            w.next();
            const int ya = y0 + 2 * cs[u], yb = ya + 1;
            const bool in = cs[u] < NC && zs[u] < nz;
            ia[u] = ((size_t)x * ny + ya) * nz + zs[u];
            oka[u] = in && ya < ny && SC_IDX_OK(st, code, ia[u], ncell);
            okb[u] = in && yb < ny && SC_IDX_OK(st, code + 1, ia[u] + nz, ncell);
        }
        R re[U], im[U];
        if (qfix) {
            long long fa[U], fb[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                fa[u] = oka[u] ? qfix[ia[u]] : 0;
                fb[u] = okb[u] ? qfix[ia[u] + nz] : 0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                re[u] = (R)(__ll2float_rn(fa[u]) * ufix);
                im[u] = (R)(__ll2float_rn(fb[u]) * ufix);
                if (oka[u]) q[ia[u]] = re[u];
                if (okb[u]) q[ia[u] + nz] = im[u];
            }
        } else {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                re[u] = oka[u] ? q[ia[u]] : (R)0;
                im[u] = okb[u] ? q[ia[u] + nz] : (R)0;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (cs[u] < NC) a[cs[u] * lz + zs[u]] = cx<R>(re[u], im[u]);
    }
}

// qfix != nullptr: the charge arrives as the 64-bit fixed-point grid of the
// FP32 form's exact deposit; it is scaled to R here and also stored in q
// (the charge grid an inspection reads back)
template <typename R>
__device__ __forceinline__ void zfwd_body(R* __restrict__ q, const long long* __restrict__ qfix,
                                          Cx<R>* __restrict__ W, int ny, int nz, int My, int Kz,
                                          const RadixPlan& rz, const Cx<R>* __restrict__ twg, int NC,
                                          const ScState* st, VBlk vb) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (st->status) return;
    const int Mz = rz.L, lz = fft_ls(Mz);
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* a = tw + Mz;
    Cx<R>* b = a + NC * lz;
    load_twiddles<R>(tw, twg, Mz);
    const int x = vb.y;
    const int y0 = vb.x * 2 * NC;
    stage_charge_lines<R>(q, qfix, a, lz, x, y0, NC, ny, nz, Mz, st, (long long)vb.ny * ny * nz, 21);
    __syncthreads();
    Cx<R>* res = fft_lines<R, false>(a, b, lz, NC, rz, tw);
    for (DivWalk w(threadIdx.x, blockDim.x, Kz); w.q < NC; w.next()) {
        const int c = w.q, k = w.r;
        const int ya = y0 + 2 * c, yb = ya + 1;
        const Cx<R> Z = res[c * lz + k];
        const Cx<R> Zm = res[c * lz + (k == 0 ? 0 : Mz - k)];
        const R h = (R)0.5;
        if (!SC_IDX_OK(st, 24, ((long long)x * My + (yb < ny ? yb : ya)) * Kz + k, (long long)vb.ny * My * Kz)) continue;
        if (ya < ny) W[((size_t)x * My + ya) * Kz + k] = cx<R>((Z.x + Zm.x) * h, (Z.y - Zm.y) * h);
        if (yb < ny) W[((size_t)x * My + yb) * Kz + k] = cx<R>((Z.y + Zm.y) * h, (Zm.x - Z.x) * h);
    }
}

template <typename R>
__global__ void __launch_bounds__(FFT_THREADS) k_zfwd(R* __restrict__ q, const long long* __restrict__ qfix,
                                                      Cx<R>* __restrict__ W, int ny, int nz, int My, int Kz,
                                                      RadixPlan rz, const Cx<R>* __restrict__ twg, int NC,
                                                      const ScState* st) {
    pdl_wait();
    zfwd_body<R>(q, qfix, W, ny, nz, My, Kz, rz, twg, NC, st, hw_vblk());
}

// strided pass along y: forward (rows < ny in, all My out) or inverse (all in, rows < ny out),
// in place on W.  The columns are the nx * Kz lines (x, kz), flattened as
// x * Kz + kz; block vb.x takes TK consecutive ones (a block may straddle two
// x planes).  W3 != nullptr (inverse, spectral fields): the block also
// transforms its columns of W multiplied by D(ky) into W3 (a third line buffer)
template <typename R, bool INV>
__device__ __forceinline__ void ypass_body(Cx<R>* __restrict__ W, int nx, int ny, int My, int Kz, const RadixPlan& ry,
                                           const Cx<R>* __restrict__ twg, int TK, const ScState* st, VBlk vb,
                                           Cx<R>* __restrict__ W3 = nullptr, const Cx<R>* __restrict__ dy = nullptr) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (st->status) return;
    const int ls = fft_ls(My);
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* a = tw + My;
    Cx<R>* b = a + TK * ls;
    Cx<R>* c = b + TK * ls;
    load_twiddles<R>(tw, twg, My);
    const ColMap cm(TK);
    const int col = vb.x * TK + cm.kk;
    const bool live = col < nx * Kz;
    const int x = col / Kz, k = col - x * Kz;
    const size_t base = ((size_t)x * My) * Kz + k;  // element y of the column at base + y * Kz
    const int nin = INV ? My : ny;
    Cx<R>* la = a + cm.kk * ls;
    Cx<R>* lc = c + cm.kk * ls;
    constexpr int U = 8;  // rows per round: their loads are issued together
    for (int y0 = cm.r0; y0 < My; y0 += U * cm.rs) {
        Cx<R> v[U], d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int y = y0 + u * cm.rs;
            v[u] = (y < nin && live) ? W[base + (size_t)y * Kz] : cx<R>(0, 0);
            d[u] = (W3 && y < My) ? dy[y] : cx<R>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int y = y0 + u * cm.rs;
            if (y < My) {
                la[y] = v[u];
                if (W3) lc[y] = cmul(v[u], d[u]);
            }
        }
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, INV>(a, b, ls, TK, ry, tw);
    const int nout = INV ? ny : My;
    if (live)
        for (int y = cm.r0; y < nout; y += cm.rs) W[base + (size_t)y * Kz] = res[cm.kk * ls + y];
    if (W3) {
        __syncthreads();  // a and b are free
        Cx<R>* res3 = fft_lines<R, INV>(c, a, ls, TK, ry, tw);
        if (live)
            for (int y = cm.r0; y < nout; y += cm.rs) W3[base + (size_t)y * Kz] = res3[cm.kk * ls + y];
    }
}

// blockIdx.y = 0: W (and, with spectral fields, W x D(ky) into W3);
// blockIdx.y = 1 (inverse, spectral fields): the x-differenced grid W2 in place
template <typename R, bool INV>
__global__ void __launch_bounds__(FFT_THREADS) k_ypass(Cx<R>* __restrict__ W, int nx, int ny, int My, int Kz,
                                                       RadixPlan ry, const Cx<R>* __restrict__ twg,
                                                       int TK, const ScState* st, Spec<R> sp) {
    pdl_wait();
    if (blockIdx.y == 0) ypass_body<R, INV>(W, nx, ny, My, Kz, ry, twg, TK, st, hw_vblk(), sp.W3, sp.dy);
    else ypass_body<R, INV>(sp.W2, nx, ny, My, Kz, ry, twg, TK, st, hw_vblk());
}

// x pass: forward FFT of the nx non-zero planes, Green multiply, inverse FFT, keep x < nx.
// The columns are the My * Kz lines (ky, kz), flattened as ky * Kz + kz (the
// element x of a column at x * My * Kz + column); block vb.x takes TK
// consecutive ones.  W2 != nullptr (spectral fields): the product times D(kx)
// goes through its own inverse transform (a third line buffer) into W2
template <typename R>
__device__ __forceinline__ void xconv_body(Cx<R>* __restrict__ W, const R* __restrict__ G, int nx, int My, int Kz,
                                           int Ky, const RadixPlan& rx, const Cx<R>* __restrict__ twg, int TK,
                                           const ScState* st, VBlk vb, Cx<R>* __restrict__ W2 = nullptr,
                                           const Cx<R>* __restrict__ dx = nullptr) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (st->status) return;
    const int Mx = rx.L;
    const int ls = fft_ls(Mx);
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* a = tw + Mx;
    Cx<R>* b = a + TK * ls;
    Cx<R>* c = b + TK * ls;
    load_twiddles<R>(tw, twg, Mx);
    const ColMap cm(TK);
    const int col = vb.x * TK + cm.kk;
    const int ncol = My * Kz;
    const bool live = col < ncol;
    const int ky = col / Kz, k = col - ky * Kz;
    const int gy = ky <= My - ky ? ky : My - ky;
    const int gk = gy * Kz + k;  // the column's Green entry at gx * Ky * Kz + gk
    const int KyKz = Ky * Kz;
    Cx<R>* la = a + cm.kk * ls;
    constexpr int U = 8;  // rows per round: their loads are issued together
    for (int x0 = cm.r0; x0 < Mx; x0 += U * cm.rs) {
        Cx<R> v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int x = x0 + u * cm.rs;
            v[u] = (x < nx && live) ? W[(size_t)x * ncol + col] : cx<R>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (x0 + u * cm.rs < Mx) la[x0 + u * cm.rs] = v[u];
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, false>(a, b, ls, TK, rx, tw);
    Cx<R>* lr = res + cm.kk * ls;
    Cx<R>* lc = c + cm.kk * ls;
    for (int x0 = cm.r0; x0 < Mx; x0 += U * cm.rs) {
        R g[U];
        Cx<R> d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int kx = x0 + u * cm.rs;
            const int gx = kx <= Mx - kx ? kx : Mx - kx;
            const long long gi = (long long)gx * KyKz + gk;
            g[u] = (kx < Mx && live && SC_IDX_OK(st, 23, gi, (long long)(rx.L / 2 + 1) * KyKz)) ? G[gi] : (R)0;
            d[u] = (W2 && kx < Mx) ? dx[kx] : cx<R>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int kx = x0 + u * cm.rs;
            if (kx < Mx) {
                Cx<R> v = lr[kx];
                v.x *= g[u];
                v.y *= g[u];
                lr[kx] = v;
                if (W2) lc[kx] = cmul(v, d[u]);
            }
        }
    }
    __syncthreads();
    Cx<R>* res2 = fft_lines<R, true>(res, res == a ? b : a, ls, TK, rx, tw);
    if (live)
        for (int x = cm.r0; x < nx; x += cm.rs) W[(size_t)x * ncol + col] = res2[cm.kk * ls + x];
    if (W2) {
        __syncthreads();  // a and b are free
        Cx<R>* res3 = fft_lines<R, true>(c, a, ls, TK, rx, tw);
        if (live)
            for (int x = cm.r0; x < nx; x += cm.rs) W2[(size_t)x * ncol + col] = res3[cm.kk * ls + x];
    }
}

template <typename R>
__global__ void __launch_bounds__(FFT_THREADS) k_xconv(Cx<R>* __restrict__ W, const R* __restrict__ G,
                                                       int nx, int My, int Kz, int Ky, RadixPlan rx,
                                                       const Cx<R>* __restrict__ twg, int TK, const ScState* st,
                                                       Spec<R> sp) {
    pdl_wait();
    xconv_body<R>(W, G, nx, My, Kz, Ky, rx, twg, TK, st, hw_vblk(), sp.W2, sp.dx);
}

// Field outputs of the inverse passes (spectral fields, FP32): the grid a
// block writes, D(kz) applied before the z inverse or not, the factor 1/h of
// the difference and the plane left at zero (sc.py:196-198).
struct InvOut {
    int field;   // 0 potential, 1 Ex, 2 Ey, 3 Ez
    int nx;
};
template <typename R>
__device__ __forceinline__ void inv_out(const Spec<R>& sp, const ScState* st, int f, const Cx<R>* W, R* phi,
                                        const Cx<R>*& src, R*& out, const Cx<R>*& dz, R& mul) {
    src = f == 1 ? sp.W2 : (f == 2 && sp.W3 ? sp.W3 : W);
    out = f == 0 ? phi : (f == 1 ? sp.ex : (f == 2 ? sp.ey : sp.ez));
    dz = f == 3 ? sp.dz : nullptr;
    mul = f == 0 ? (R)1 : (R)st->istepsf[f - 1];
}

// dz != nullptr: the z spectrum is multiplied by D(kz) first; mul scales the
// output; zero_axis (0, 1, 2) leaves the last plane along that axis at zero
// (x = nx - 1, y = ny - 1 or z = nz - 1), -1 none
template <typename R>
__device__ __forceinline__ void zinv_body(const Cx<R>* __restrict__ W, R* __restrict__ phi, int ny, int nz, int My,
                                          int Kz, const RadixPlan& rz, const Cx<R>* __restrict__ twg, int NC,
                                          const ScState* st, VBlk vb, const Cx<R>* __restrict__ dz = nullptr,
                                          R mul = (R)1, int zero_axis = -1, int nx = 0) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (st->status) return;
    const int Mz = rz.L, lz = fft_ls(Mz);
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* a = tw + Mz;
    Cx<R>* b = a + NC * lz;
    load_twiddles<R>(tw, twg, Mz);
    const int x = vb.y;
    const int y0 = vb.x * 2 * NC;
    constexpr int U = 4;  // elements per thread per round, their loads issued together
    for (DivWalk w(threadIdx.x, blockDim.x, Mz); w.q < NC;) {
        int cs[U], ks[U];
        Cx<R> A[U], B[U], d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            cs[u] = w.q;
            ks[u] = w.r;
            w.next();
            const int ya = y0 + 2 * cs[u], yb = ya + 1;
            const bool in = cs[u] < NC;
            const int kk = ks[u] < Kz ? ks[u] : Mz - ks[u];
            A[u] = (in && ya < ny) ? W[((size_t)x * My + ya) * Kz + kk] : cx<R>(0, 0);
            B[u] = (in && yb < ny) ? W[((size_t)x * My + yb) * Kz + kk] : cx<R>(0, 0);
            d[u] = (dz && in) ? dz[kk] : cx<R>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (cs[u] >= NC) continue;
            Cx<R> Au = A[u], Bu = B[u];
            if (dz) {
                Au = cmul(Au, d[u]);
                Bu = cmul(Bu, d[u]);
            }
            // Z = A + iB, Hermitian-extended above Mz/2
            a[cs[u] * lz + ks[u]] = ks[u] < Kz ? cx<R>(Au.x - Bu.y, Au.y + Bu.x) : cx<R>(Au.x + Bu.y, Bu.x - Au.y);
        }
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, true>(a, b, lz, NC, rz, tw);
    const double norm = st->phi_norm, denom = st->phi_denom;
    const R fscale = (R)st->phi_scalef * mul;  // (float)(norm / denom), computed once by the mesh finalize
    for (DivWalk w(threadIdx.x, blockDim.x, nz); w.q < NC; w.next()) {
        const int c = w.q, z = w.r;
        const int ya = y0 + 2 * c, yb = ya + 1;
        const Cx<R> v = res[c * lz + z];
        if (sizeof(R) == 8) {
            // out/(4*pi*eps0*hx*hy*hz) after the 1/M normalisation of ifftn (sc.py:164-167)
            if (ya < ny) phi[((size_t)x * ny + ya) * nz + z] = (R)(((double)v.x * norm) / denom);
            if (yb < ny) phi[((size_t)x * ny + yb) * nz + z] = (R)(((double)v.y * norm) / denom);
        } else {
            const bool zx = zero_axis == 0 && x == nx - 1, zz = zero_axis == 2 && z == nz - 1;
            const bool za = zx || zz || (zero_axis == 1 && ya == ny - 1);
            const bool zb = zx || zz || (zero_axis == 1 && yb == ny - 1);
            if (ya < ny) phi[((size_t)x * ny + ya) * nz + z] = za ? (R)0 : v.x * fscale;
            if (yb < ny) phi[((size_t)x * ny + yb) * nz + z] = zb ? (R)0 : v.y * fscale;
        }
    }
}

// blockIdx.z: the output (0 the potential; with spectral fields 1 Ex, 2 Ey, 3 Ez)
template <typename R>
__global__ void __launch_bounds__(FFT_THREADS) k_zinv(const Cx<R>* __restrict__ W, R* __restrict__ phi,
                                                      int ny, int nz, int My, int Kz, RadixPlan rz,
                                                      const Cx<R>* __restrict__ twg, int NC,
                                                      const ScState* st, Spec<R> sp) {
    pdl_wait();
    const int f = (int)blockIdx.z + sp.f0;
    const Cx<R>* src;
    R* out;
    const Cx<R>* dz;
    R mul;
    inv_out<R>(sp, st, f, W, phi, src, out, dz, mul);
    zinv_body<R>(src, out, ny, nz, My, Kz, rz, twg, NC, st, hw_vblk(), dz, mul, f - 1, (int)gridDim.y);
}

// Ex,Ey,Ez = forward differences / h, zero on the last plane (sc.py:195-200).
// One block per (x, y) line of cells, one thread per z: no index division.
template <typename R>
__global__ void k_field_grids(const R* __restrict__ phi, R* __restrict__ ex, R* __restrict__ ey,
                              R* __restrict__ ez, int nx, int ny, int nz, const ScState* st) {
    pdl_wait();
    if (st->status) return;
    const int j = blockIdx.x, i = blockIdx.y;
    const double hx = st->steps[0], hy = st->steps[1], hz = st->steps[2];
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        const int c = (i * ny + j) * nz + k;
        const R p = phi[c];
        R vx = 0, vy = 0, vz = 0;
        if (i < nx - 1) vx = (R)(((double)p - (double)phi[c + ny * nz]) / hx);
        if (j < ny - 1) vy = (R)(((double)p - (double)phi[c + nz]) / hy);
        if (k < nz - 1) vz = (R)(((double)p - (double)phi[c + 1]) / hz);
        ex[c] = vx;
        ey[c] = vy;
        ez[c] = vz;
    }
}

// FP32 form: the field grids as "octs" for the gather -- for each cell
// (i,j,k) and each component F, the 8 values F[i+a][j+b][k+c] (a, b, c in
// {0,1}) at index 4a + 2b + c, 32 bytes aligned to 32; a trilinear sample
// then reads one 32-byte sector instead of eight scalars.  Entries that the
// gather never uses (i = nx-1, j = ny-1 or k = nz-1 as a base) are written
// but not read.
__device__ __forceinline__ float fd(const float* __restrict__ phi, int i, int j, int k, int di, int dj, int dk,
                                    int nx, int ny, int nz, float ih) {
    // forward difference along (di,dj,dk), zero on the last plane and outside the grid
    if (i >= nx || j >= ny || k >= nz) return 0.f;
    if (i + di >= nx || j + dj >= ny || k + dk >= nz) return 0.f;
    const int c = (i * ny + j) * nz + k;
    return (phi[c] - phi[c + (di * ny + dj) * nz + dk]) * ih;
}

__device__ __forceinline__ void st_oct(float* p, const float (&o)[8]) {
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(o[0]), "f"(o[1]), "f"(o[2]),
                 "f"(o[3]), "f"(o[4]), "f"(o[5]), "f"(o[6]), "f"(o[7])
                 : "memory");
}

__device__ __forceinline__ void field_octs_body(const float* __restrict__ phi, float* __restrict__ ox,
                                                float* __restrict__ oy, float* __restrict__ oz, int nx, int ny,
                                                int nz, const ScState* st, VBlk vb) {
    if (st->status) return;
    const int j = vb.x, i = vb.y;
    const float ih[3] = {st->istepsf[0], st->istepsf[1], st->istepsf[2]};
    float* const out[3] = {ox, oy, oz};
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        const size_t c = ((size_t)i * ny + j) * nz + k;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float o[8];
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b)
#pragma unroll
                    for (int e = 0; e < 2; ++e)
                        o[4 * a + 2 * b + e] = fd(phi, i + a, j + b, k + e, d == 0, d == 1, d == 2, nx, ny, nz, ih[d]);
            st_oct(out[d] + 8 * c, o);
        }
    }
}

__global__ void k_field_octs(const float* __restrict__ phi, float* __restrict__ ox, float* __restrict__ oy,
                             float* __restrict__ oz, int nx, int ny, int nz, const ScState* st) {
    pdl_wait();
    field_octs_body(phi, ox, oy, oz, nx, ny, nz, st, hw_vblk());
}

// the octs of field grids computed in Fourier space (spectral fields): the 8
// neighbouring values themselves, zero outside the grid
__device__ __forceinline__ float at_or0(const float* __restrict__ F, int i, int j, int k, int nx, int ny, int nz) {
    return (i < nx && j < ny && k < nz) ? F[((size_t)i * ny + j) * nz + k] : 0.f;
}
__device__ __forceinline__ void field_octs_spectral_body(const float* __restrict__ ex, const float* __restrict__ ey,
                                                         const float* __restrict__ ez, float* __restrict__ ox,
                                                         float* __restrict__ oy, float* __restrict__ oz, int nx,
                                                         int ny, int nz, const ScState* st, VBlk vb) {
    if (st->status) return;
    const int j = vb.x, i = vb.y;
    const float* const in[3] = {ex, ey, ez};
    float* const out[3] = {ox, oy, oz};
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {
        const size_t c = ((size_t)i * ny + j) * nz + k;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float o[8];
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b)
#pragma unroll
                    for (int e = 0; e < 2; ++e) o[4 * a + 2 * b + e] = at_or0(in[d], i + a, j + b, k + e, nx, ny, nz);
            st_oct(out[d] + 8 * c, o);
        }
    }
}
__global__ void k_field_octs_spectral(const float* __restrict__ ex, const float* __restrict__ ey,
                                      const float* __restrict__ ez, float* __restrict__ ox, float* __restrict__ oy,
                                      float* __restrict__ oz, int nx, int ny, int nz, const ScState* st) {
    pdl_wait();
    field_octs_spectral_body(ex, ey, ez, ox, oy, oz, nx, ny, nz, st, hw_vblk());
}


// ---------------------------------------------------------------------------
// Plane-fused passes (meshes whose y-by-kz plane fits in shared memory): one
// block per x plane does the z and y forward transforms (F1 + F2), or the y
// and z inverse transforms (B2 + B1), keeping the plane in shared memory
// between them.  The lines go through the same fft_lines code as the
// separate passes, so the results are identical; the plane saves a kernel
// launch and a round trip of the work grid per direction.
// Shared memory: twiddles z and y, then two buffers of Kz y-lines; the z
// lines use the second buffer (forward) or whichever buffer the y result
// does not occupy (inverse).
// ---------------------------------------------------------------------------
constexpr int PLANE_THREADS = 1024;

template <typename R>
static size_t plane_smem(const Plan& p) {
    const int Kz = p.Mz / 2 + 1;
    return sizeof(Cx<R>) * ((size_t)p.Mz + p.My + 2 * (size_t)Kz * fft_ls(p.My));
}
template <typename R>
static bool plane_fits(const Plan& p, int optin) {
    const int Kz = p.Mz / 2 + 1, ncz = (p.ny + 1) / 2;
    return 2 * (size_t)ncz * fft_ls(p.Mz) <= (size_t)Kz * fft_ls(p.My) && plane_smem<R>(p) <= (size_t)optin;
}

template <typename R>
__device__ __forceinline__ void zy_fwd_body(R* __restrict__ q, const long long* __restrict__ qfix,
                                            Cx<R>* __restrict__ W, int ny, int nz, int My, int Kz,
                                            const RadixPlan& rz, const RadixPlan& ry, const Cx<R>* __restrict__ twzg,
                                            const Cx<R>* __restrict__ twyg, const ScState* st, int x, int nx) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (st->status) return;
    const int Mz = rz.L, lz = fft_ls(Mz), ly = fft_ls(My), ncz = (ny + 1) / 2;
    Cx<R>* twz = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* twy = twz + Mz;
    Cx<R>* A2 = twy + My;
    Cx<R>* B2 = A2 + Kz * ly;
    Cx<R>* A1 = B2;
    Cx<R>* B1 = A1 + ncz * lz;
    load_twiddles<R>(twz, twzg, Mz);
    load_twiddles<R>(twy, twyg, My);
    // F1: two charge rows per complex line (as k_zfwd)
    stage_charge_lines<R>(q, qfix, A1, lz, x, 0, ncz, ny, nz, Mz, st, (long long)nx * ny * nz, 25);
    __syncthreads();
    const Cx<R>* res1 = fft_lines<R, false>(A1, B1, lz, ncz, rz, twz);
    // unpack the two real lines into the y lines (column kz, row y); rows
    // ny..My-1 are the zero padding of F2
    for (DivWalk w(threadIdx.x, blockDim.x, Kz); w.q < ncz; w.next()) {
        const int c = w.q, k = w.r;
        const int ya = 2 * c, yb = ya + 1;
        const Cx<R> Z = res1[c * lz + k];
        const Cx<R> Zm = res1[c * lz + (k == 0 ? 0 : Mz - k)];
        const R h = (R)0.5;
        A2[k * ly + ya] = cx<R>((Z.x + Zm.x) * h, (Z.y - Zm.y) * h);
        if (yb < ny) A2[k * ly + yb] = cx<R>((Z.y + Zm.y) * h, (Zm.x - Z.x) * h);
    }
    for (DivWalk w(threadIdx.x, blockDim.x, Kz); w.q < My - ny; w.next()) A2[w.r * ly + ny + w.q] = cx<R>(0, 0);
    __syncthreads();
    const Cx<R>* res2 = fft_lines<R, false>(A2, B2, ly, Kz, ry, twy);
    Cx<R>* Wx = W + (size_t)x * My * Kz;  // the plane: row ky, column k at ky * Kz + k
    for (DivWalk w(threadIdx.x, blockDim.x, Kz); w.q < My; w.next()) Wx[w.q * Kz + w.r] = res2[w.r * ly + w.q];
}

template <typename R>
__global__ void __launch_bounds__(PLANE_THREADS) k_zy_fwd(R* __restrict__ q, const long long* __restrict__ qfix,
                                                          Cx<R>* __restrict__ W, int ny, int nz, int My, int Kz,
                                                          RadixPlan rz, RadixPlan ry, const Cx<R>* __restrict__ twz,
                                                          const Cx<R>* __restrict__ twy, const ScState* st) {
    pdl_wait();
    zy_fwd_body<R>(q, qfix, W, ny, nz, My, Kz, rz, ry, twz, twy, st, (int)blockIdx.x, (int)gridDim.x);
}

// dy / dz != nullptr (spectral fields): the plane is multiplied by D(ky)
// before the y inverse / by D(kz) before the z inverse; mul and zero_axis as
// in zinv_body
template <typename R>
__device__ __forceinline__ void yz_inv_body(const Cx<R>* __restrict__ W, R* __restrict__ phi, int ny, int nz,
                                            int My, int Kz, const RadixPlan& rz, const RadixPlan& ry,
                                            const Cx<R>* __restrict__ twzg, const Cx<R>* __restrict__ twyg,
                                            const ScState* st, int x, const Cx<R>* __restrict__ dy = nullptr,
                                            const Cx<R>* __restrict__ dz = nullptr, R mul = (R)1,
                                            int zero_axis = -1, int nx = 0) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (st->status) return;
    const int Mz = rz.L, lz = fft_ls(Mz), ly = fft_ls(My), ncz = (ny + 1) / 2;
    Cx<R>* twz = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* twy = twz + Mz;
    Cx<R>* A2 = twy + My;
    Cx<R>* B2 = A2 + Kz * ly;
    load_twiddles<R>(twz, twzg, Mz);
    load_twiddles<R>(twy, twyg, My);
    const Cx<R>* Wx = W + (size_t)x * My * Kz;
    constexpr int U = 4;  // elements per thread per round, their loads issued together
    for (DivWalk w(threadIdx.x, blockDim.x, Kz); w.q < My;) {
        int ys[U], ks[U];
        Cx<R> v[U], d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            ys[u] = w.q;
            ks[u] = w.r;
            w.next();
            const bool in = ys[u] < My;
            v[u] = in ? Wx[ys[u] * Kz + ks[u]] : cx<R>(0, 0);
            d[u] = (dy && in) ? dy[ys[u]] : cx<R>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (ys[u] < My) A2[ks[u] * ly + ys[u]] = dy ? cmul(v[u], d[u]) : v[u];
    }
    __syncthreads();
    // B2: inverse y; only rows y < ny are used
    const Cx<R>* res2 = fft_lines<R, true>(A2, B2, ly, Kz, ry, twy);
    Cx<R>* A1 = res2 == B2 ? A2 : B2;
    Cx<R>* B1 = A1 + ncz * lz;
    // B1: two output rows per complex line, Hermitian-extended (as k_zinv)
    for (DivWalk w(threadIdx.x, blockDim.x, Mz); w.q < ncz; w.next()) {
        const int c = w.q, k = w.r;
        const int ya = 2 * c, yb = ya + 1;
        const bool lo = k < Kz;
        const int kk = lo ? k : Mz - k;
        Cx<R> A = res2[kk * ly + ya];
        Cx<R> B = yb < ny ? res2[kk * ly + yb] : cx<R>(0, 0);
        if (dz) {
            A = cmul(A, dz[kk]);
            B = cmul(B, dz[kk]);
        }
        A1[c * lz + k] = lo ? cx<R>(A.x - B.y, A.y + B.x) : cx<R>(A.x + B.y, B.x - A.y);
    }
    __syncthreads();
    const Cx<R>* res = fft_lines<R, true>(A1, B1, lz, ncz, rz, twz);
    const double norm = st->phi_norm, denom = st->phi_denom;
    const R fscale = (R)st->phi_scalef * mul;  // (float)(norm / denom), computed once by the mesh finalize
    for (DivWalk w(threadIdx.x, blockDim.x, nz); w.q < ncz; w.next()) {
        const int c = w.q, z = w.r;
        const int ya = 2 * c, yb = ya + 1;
        const Cx<R> v = res[c * lz + z];
        if (sizeof(R) == 8) {
            // out/(4*pi*eps0*hx*hy*hz) after the 1/M normalisation of ifftn (sc.py:164-167)
            phi[((size_t)x * ny + ya) * nz + z] = (R)(((double)v.x * norm) / denom);
            if (yb < ny) phi[((size_t)x * ny + yb) * nz + z] = (R)(((double)v.y * norm) / denom);
        } else {
            const bool zx = zero_axis == 0 && x == nx - 1, zz = zero_axis == 2 && z == nz - 1;
            const bool za = zx || zz || (zero_axis == 1 && ya == ny - 1);
            const bool zb = zx || zz || (zero_axis == 1 && yb == ny - 1);
            phi[((size_t)x * ny + ya) * nz + z] = za ? (R)0 : v.x * fscale;
            if (yb < ny) phi[((size_t)x * ny + yb) * nz + z] = zb ? (R)0 : v.y * fscale;
        }
    }
}

// blockIdx.y: the output (0 the potential; with spectral fields 1 Ex, 2 Ey, 3 Ez)
template <typename R>
__global__ void __launch_bounds__(PLANE_THREADS) k_yz_inv(const Cx<R>* __restrict__ W, R* __restrict__ phi, int ny,
                                                          int nz, int My, int Kz, RadixPlan rz, RadixPlan ry,
                                                          const Cx<R>* __restrict__ twz,
                                                          const Cx<R>* __restrict__ twy, const ScState* st,
                                                          Spec<R> sp) {
    pdl_wait();
    const int f = (int)blockIdx.y + sp.f0;
    const Cx<R>* src;
    R* out;
    const Cx<R>* dz;
    R mul;
    Spec<R> spp = sp;
    spp.W3 = nullptr;  // the plane pass applies D(ky) itself
    inv_out<R>(spp, st, f, W, phi, src, out, dz, mul);
    yz_inv_body<R>(src, out, ny, nz, My, Kz, rz, ry, twz, twy, st, (int)blockIdx.x, f == 2 ? sp.dy : nullptr, dz,
                   mul, f - 1, (int)gridDim.x);
}

static int optin_smem();
// the plane-fused passes are used where the plane fits shared memory and the
// plan's parameters (SC_PARAM_FFT_PLANE_FWD / _INV) allow them
static bool plane_ok(const Plan& p) {
    return p.prec == SC_FP64 ? plane_fits<double>(p, optin_smem()) : plane_fits<float>(p, optin_smem());
}
int convolve_launches(const Plan& p) {
    const bool plane = plane_ok(p);
    return (plane && p.fft_plane_fwd ? 1 : 2) + 1 + (plane && p.fft_plane_inv ? 1 : 2);
}

static int optin_smem() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) || cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) return 0;
    return v;
}

// the spectral-field pointers of a plan's workspace (W2 == nullptr: none)
// want_phi: the inverse passes also produce the potential (the kick's field
// octs do not read it; an inspection or the record-field mode does)
template <typename R>
__host__ __device__ __forceinline__ Spec<R> spec_of(const Plan& p, const Layout& L, char* ws, bool fields,
                                                    bool want_phi = true) {
    Spec<R> sp = {};
    if (!(fields && p.spectral && sizeof(R) == 4)) return sp;
    sp.f0 = want_phi ? 0 : 1;
    sp.W2 = reinterpret_cast<Cx<R>*>(ws + L.W2);
    sp.W3 = reinterpret_cast<Cx<R>*>(ws + L.W3);
    sp.dx = reinterpret_cast<const Cx<R>*>(ws + L.dt_x);
    sp.dy = reinterpret_cast<const Cx<R>*>(ws + L.dt_y);
    sp.dz = reinterpret_cast<const Cx<R>*>(ws + L.dt_z);
    sp.ex = reinterpret_cast<R*>(ws + L.ex);
    sp.ey = reinterpret_cast<R*>(ws + L.ey);
    sp.ez = reinterpret_cast<R*>(ws + L.ez);
    return sp;
}

template <typename R>
static cudaError_t convolve_t(const Plan& p, const Layout& L, char* ws, R* qgrid, R* phi, const long long* qfix,
                              cudaStream_t s, int part, bool fields, bool want_phi) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int Kz = p.Mz / 2 + 1, Ky = p.My / 2 + 1;
    const Spec<R> sp = spec_of<R>(p, L, ws, fields, want_phi);
    const int nbuf = sp.W2 ? 3 : 2;  // line buffers of the x pass and the y inverse
    Cx<R>* W = reinterpret_cast<Cx<R>*>(ws + L.W);
    const R* G = reinterpret_cast<const R*>(ws + L.green);
    const Cx<R>* twx = reinterpret_cast<const Cx<R>*>(ws + L.tw_x);
    const Cx<R>* twy = reinterpret_cast<const Cx<R>*>(ws + L.tw_y);
    const Cx<R>* twz = reinterpret_cast<const Cx<R>*>(ws + L.tw_z);
    cudaError_t e;
    const int NC = z_lines_per_block(p.Mz);
    const size_t smz = sizeof(Cx<R>) * (size_t)(p.Mz + 2 * NC * fft_ls(p.Mz));
    dim3 gz((p.ny + 2 * NC - 1) / (2 * NC), p.nx);
    const int tky = pass_cols<R>(p.fft_cols_y, p.My), tkx = pass_cols<R>(p.fft_cols_x, p.Mx, nbuf);
    const int tkyi = pass_cols<R>(p.fft_cols_y, p.My, nbuf);  // the y inverse
    const size_t smy = sizeof(Cx<R>) * (size_t)(p.My + 2 * tky * fft_ls(p.My));
    const size_t smyi = sizeof(Cx<R>) * (size_t)(p.My + nbuf * tkyi * fft_ls(p.My));
    const int ycols = p.nx * Kz;  // the y passes' columns (x, kz)
    dim3 gy((ycols + tky - 1) / tky);
    dim3 gyi((ycols + tkyi - 1) / tkyi, sp.W2 ? 2 : 1);
    static const int optin = optin_smem();
    const bool plane = plane_fits<R>(p, optin);
    const bool plane_fwd = plane && p.fft_plane_fwd, plane_inv = plane && p.fft_plane_inv;
    const size_t smp = plane_smem<R>(p);
    if (plane_fwd && part != CONV_REST) {
        if ((e = set_smem(k_zy_fwd<R>, smp))) return e;
        launch(k_zy_fwd<R>, p.nx, PLANE_THREADS, smp, s, qgrid, qfix, W, p.ny, p.nz, p.My, Kz, p.rz, p.ry, twz, twy, st);
    } else if (part != CONV_REST) {
        if ((e = set_smem(k_zfwd<R>, smz))) return e;
        launch(k_zfwd<R>, gz, FFT_THREADS, smz, s, qgrid, qfix, W, p.ny, p.nz, p.My, Kz, p.rz, twz, NC, st);
        if ((e = set_smem(k_ypass<R, false>, smy))) return e;
        launch(k_ypass<R, false>, gy, FFT_THREADS, smy, s, W, p.nx, p.ny, p.My, Kz, p.ry, twy, tky, st, Spec<R>{});
    }
    if (part == CONV_FORWARD) return cudaGetLastError();
    const size_t smx = sizeof(Cx<R>) * (size_t)(p.Mx + nbuf * tkx * fft_ls(p.Mx));
    dim3 gx((p.My * Kz + tkx - 1) / tkx);  // the x pass's columns (ky, kz)
    if ((e = set_smem(k_xconv<R>, smx))) return e;
    launch(k_xconv<R>, gx, FFT_THREADS, smx, s, W, G, p.nx, p.My, Kz, Ky, p.rx, twx, tkx, st, sp);
    const int nout = sp.W2 ? 4 - sp.f0 : 1;  // [the potential,] Ex, Ey, Ez
    if (plane_inv) {
        if ((e = set_smem(k_yz_inv<R>, smp))) return e;
        launch(k_yz_inv<R>, dim3(p.nx, nout), PLANE_THREADS, smp, s, W, phi, p.ny, p.nz, p.My, Kz, p.rz, p.ry, twz, twy,
               st, sp);
        return cudaGetLastError();
    }
    if ((e = set_smem(k_ypass<R, true>, smyi))) return e;
    launch(k_ypass<R, true>, gyi, FFT_THREADS, smyi, s, W, p.nx, p.ny, p.My, Kz, p.ry, twy, tkyi, st, sp);
    if ((e = set_smem(k_zinv<R>, smz))) return e;
    launch(k_zinv<R>, dim3(gz.x, gz.y, nout), FFT_THREADS, smz, s, W, phi, p.ny, p.nz, p.My, Kz, p.rz, twz, NC, st, sp);
    return cudaGetLastError();
}

template <typename R>
static cudaError_t prepare_fft_t(const Plan& p) {
    cudaError_t e;
    const int NC = z_lines_per_block(p.Mz);
    const size_t smz = sizeof(Cx<R>) * (size_t)(p.Mz + 2 * NC * fft_ls(p.Mz));
    const int nbuf = (p.spectral && sizeof(R) == 4) ? 3 : 2;
    const int tky = strided_cols<R>(p.My), tkx = strided_cols<R>(p.Mx, nbuf), tkyi = strided_cols<R>(p.My, nbuf);
    const size_t smy = sizeof(Cx<R>) * (size_t)(p.My + 2 * tky * fft_ls(p.My));
    const size_t smyi = sizeof(Cx<R>) * (size_t)(p.My + nbuf * tkyi * fft_ls(p.My));
    const size_t smx = sizeof(Cx<R>) * (size_t)(p.Mx + nbuf * tkx * fft_ls(p.Mx));
    if ((e = set_smem(k_zfwd<R>, smz))) return e;
    if ((e = set_smem(k_ypass<R, false>, smy))) return e;
    if ((e = set_smem(k_xconv<R>, smx))) return e;
    if ((e = set_smem(k_ypass<R, true>, smyi))) return e;
    if ((e = set_smem(k_zinv<R>, smz))) return e;
    if (plane_fits<R>(p, optin_smem())) {
        if ((e = set_smem(k_zy_fwd<R>, plane_smem<R>(p)))) return e;
        if ((e = set_smem(k_yz_inv<R>, plane_smem<R>(p)))) return e;
    }
    return cudaSuccess;
}

cudaError_t prepare_fft_kernels(const Plan& p) {
    return p.prec == SC_FP64 ? prepare_fft_t<double>(p) : prepare_fft_t<float>(p);
}

cudaError_t launch_convolve(const Plan& p, const Layout& L, char* ws, const void* qgrid_in, void* phi_out,
                            cudaStream_t s, const long long* qfix, int part, bool fields, bool want_phi) {
    if (p.prec == SC_FP64)
        return convolve_t<double>(p, L, ws, static_cast<double*>(const_cast<void*>(qgrid_in)),
                                  static_cast<double*>(phi_out), nullptr, s, part, false, true);
    return convolve_t<float>(p, L, ws, static_cast<float*>(const_cast<void*>(qgrid_in)), static_cast<float*>(phi_out),
                             qfix, s, part, fields, want_phi);
}

template <typename R>
static cudaError_t field_t(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int bt = p.nz < 256 ? ((p.nz + 31) / 32) * 32 : 256;
    const dim3 grid(p.ny, p.nx);
    if (sizeof(R) == 4 && p.spectral)
        launch(k_field_octs_spectral, grid, bt, 0, s, reinterpret_cast<const float*>(ws + L.ex),
               reinterpret_cast<const float*>(ws + L.ey), reinterpret_cast<const float*>(ws + L.ez),
               reinterpret_cast<float*>(ws + L.exq), reinterpret_cast<float*>(ws + L.eyq),
               reinterpret_cast<float*>(ws + L.ezq), p.nx, p.ny, p.nz, st);
    else if (sizeof(R) == 4)
        launch(k_field_octs, grid, bt, 0, s, reinterpret_cast<const float*>(ws + L.phi), reinterpret_cast<float*>(ws + L.exq),
                                         reinterpret_cast<float*>(ws + L.eyq), reinterpret_cast<float*>(ws + L.ezq),
                                         p.nx, p.ny, p.nz, st);
    else
        launch(k_field_grids<R>, grid, bt, 0, s, reinterpret_cast<const R*>(ws + L.phi), reinterpret_cast<R*>(ws + L.ex),
                                             reinterpret_cast<R*>(ws + L.ey), reinterpret_cast<R*>(ws + L.ez),
                                             p.nx, p.ny, p.nz, st);
    return cudaGetLastError();
}

cudaError_t launch_field_grids(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    return p.prec == SC_FP64 ? field_t<double>(p, L, ws, s) : field_t<float>(p, L, ws, s);
}

// ---------------------------------------------------------------------------
// batched convolution and field (FP32 form): one launch per pass over every
// beam of a batch, each beam with the tiling of its plain launch
// ---------------------------------------------------------------------------
#define BATCH_BEAM(stage)                                                       \
    const int b = batch_beam(start, nb);                                        \
    const BatchBeam& B = beams[b];                                              \
    const VBlk vb = batch_vblk(start, b, B.gx[stage], B.gy[stage]);             \
    char* ws = B.ws;                                                            \
    const Layout& L = B.L;                                                      \
    const Plan& p = B.p;                                                        \
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);

__global__ void __launch_bounds__(FFT_THREADS) kb_zfwd(const BatchBeam* __restrict__ beams,
                                                       const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_FFT_Z)
    zfwd_body<float>(reinterpret_cast<float*>(ws + L.qgrid), reinterpret_cast<const long long*>(ws + L.qfix),
                     reinterpret_cast<Cx<float>*>(ws + L.W), p.ny, p.nz, p.My, p.Mz / 2 + 1, p.rz,
                     reinterpret_cast<const Cx<float>*>(ws + L.tw_z), B.fft_nc, st, vb);
}

// forward y pass
__global__ void __launch_bounds__(FFT_THREADS) kb_yfwd(const BatchBeam* __restrict__ beams,
                                                       const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_FFT_Y)
    ypass_body<float, false>(reinterpret_cast<Cx<float>*>(ws + L.W), p.nx, p.ny, p.My, p.Mz / 2 + 1, p.ry,
                             reinterpret_cast<const Cx<float>*>(ws + L.tw_y), B.fft_tky, st, vb);
}

// inverse y pass: block row 0 takes W (and, with spectral fields, W x D(ky)
// into W3), row 1 the x-differenced W2 (as k_ypass's blockIdx.y)
__global__ void __launch_bounds__(FFT_THREADS) kb_yinv(const BatchBeam* __restrict__ beams,
                                                       const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_FFT_YI)
    const Spec<float> sp = spec_of<float>(p, L, ws, true);
    const Cx<float>* tw = reinterpret_cast<const Cx<float>*>(ws + L.tw_y);
    if (vb.y == 0)
        ypass_body<float, true>(reinterpret_cast<Cx<float>*>(ws + L.W), p.nx, p.ny, p.My, p.Mz / 2 + 1, p.ry, tw,
                                B.fft_tky, st, vb, sp.W3, sp.dy);
    else
        ypass_body<float, true>(sp.W2, p.nx, p.ny, p.My, p.Mz / 2 + 1, p.ry, tw, B.fft_tky, st, vb);
}

__global__ void __launch_bounds__(FFT_THREADS) kb_xconv(const BatchBeam* __restrict__ beams,
                                                        const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_FFT_X)
    const Spec<float> sp = spec_of<float>(p, L, ws, true);
    xconv_body<float>(reinterpret_cast<Cx<float>*>(ws + L.W), reinterpret_cast<const float*>(ws + L.green), p.nx,
                      p.My, p.Mz / 2 + 1, p.My / 2 + 1, p.rx, reinterpret_cast<const Cx<float>*>(ws + L.tw_x),
                      B.fft_tkx, st, vb, sp.W2, sp.dx);
}

// inverse z pass: block group f writes output f (the potential; with spectral
// fields also Ex, Ey, Ez), as k_zinv's blockIdx.z
__global__ void __launch_bounds__(FFT_THREADS) kb_zinv(const BatchBeam* __restrict__ beams,
                                                       const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_FFT_ZI)
    const Spec<float> sp = spec_of<float>(p, L, ws, true, false);
    const int f = vb.y / p.nx + sp.f0;
    const VBlk v = {vb.x, vb.y - (f - sp.f0) * p.nx, vb.nx, p.nx};
    const Cx<float>* src;
    float* out;
    const Cx<float>* dz;
    float mul;
    inv_out<float>(sp, st, f, reinterpret_cast<const Cx<float>*>(ws + L.W), reinterpret_cast<float*>(ws + L.phi), src,
                   out, dz, mul);
    zinv_body<float>(src, out, p.ny, p.nz, p.My, p.Mz / 2 + 1, p.rz, reinterpret_cast<const Cx<float>*>(ws + L.tw_z),
                     B.fft_nc, st, v, dz, mul, f - 1, p.nx);
}

__global__ void kb_field_octs(const BatchBeam* __restrict__ beams, const int* __restrict__ start, int nb) {
    pdl_wait();
    BATCH_BEAM(BS_FIELD)
    if (p.spectral)
        field_octs_spectral_body(reinterpret_cast<const float*>(ws + L.ex), reinterpret_cast<const float*>(ws + L.ey),
                                 reinterpret_cast<const float*>(ws + L.ez), reinterpret_cast<float*>(ws + L.exq),
                                 reinterpret_cast<float*>(ws + L.eyq), reinterpret_cast<float*>(ws + L.ezq), p.nx, p.ny,
                                 p.nz, st, vb);
    else
        field_octs_body(reinterpret_cast<const float*>(ws + L.phi), reinterpret_cast<float*>(ws + L.exq),
                        reinterpret_cast<float*>(ws + L.eyq), reinterpret_cast<float*>(ws + L.ezq), p.nx, p.ny, p.nz,
                        st, vb);
}
#undef BATCH_BEAM

// A batched launch gives every block the largest dynamic shared memory of
// its beams, so one beam with long lines would set the occupancy of all the
// others: the batch caps each beam's strided-pass blocks at what lets four
// blocks share an SM (228 KB per SM, 1 KB reserved per block).
constexpr size_t BATCH_FFT_SMEM = 233472 / 4 - 1024;
static int batch_cols(int tk, int M, int nbuf) {
    while (tk > 2 && sizeof(Cx<float>) * (size_t)(M + nbuf * tk * fft_ls(M)) > BATCH_FFT_SMEM) tk /= 2;
    return tk;
}

void batch_fft_tiling(BatchBeam& B, size_t smem[3]) {
    const Plan& p = B.p;
    const int Kz = p.Mz / 2 + 1;
    const int nbuf = p.spectral ? 3 : 2;  // line buffers of the x pass and the y passes
    B.fft_nc = z_lines_per_block(p.Mz);
    B.fft_tky = batch_cols(pass_cols<float>(p.fft_cols_y, p.My, nbuf), p.My, nbuf);
    B.fft_tkx = batch_cols(pass_cols<float>(p.fft_cols_x, p.Mx, nbuf), p.Mx, nbuf);
    B.gx[BS_FFT_Z] = (p.ny + 2 * B.fft_nc - 1) / (2 * B.fft_nc);
    B.gy[BS_FFT_Z] = p.nx;
    B.gx[BS_FFT_Y] = (p.nx * Kz + B.fft_tky - 1) / B.fft_tky;  // columns (x, kz)
    B.gy[BS_FFT_Y] = 1;
    B.gx[BS_FFT_X] = (p.My * Kz + B.fft_tkx - 1) / B.fft_tkx;  // columns (ky, kz)
    B.gy[BS_FFT_X] = 1;
    B.gx[BS_FFT_YI] = B.gx[BS_FFT_Y];
    B.gy[BS_FFT_YI] = p.spectral ? 2 : 1;
    B.gx[BS_FFT_ZI] = B.gx[BS_FFT_Z];
    B.gy[BS_FFT_ZI] = p.nx * (p.spectral ? 3 : 1);  // spectral fields: Ex, Ey, Ez (no potential)
    B.gx[BS_FIELD] = p.ny;
    B.gy[BS_FIELD] = p.nx;
    smem[0] = sizeof(Cx<float>) * (size_t)(p.Mz + 2 * B.fft_nc * fft_ls(p.Mz));
    smem[1] = sizeof(Cx<float>) * (size_t)(p.My + nbuf * B.fft_tky * fft_ls(p.My));
    smem[2] = sizeof(Cx<float>) * (size_t)(p.Mx + nbuf * B.fft_tkx * fft_ls(p.Mx));
}

cudaError_t prepare_batch_fft() {
    cudaError_t e;
    const size_t big = 48 * 1024 + 1;
    if ((e = smem_opt_in(reinterpret_cast<const void*>(kb_zfwd), big))) return e;
    if ((e = smem_opt_in(reinterpret_cast<const void*>(kb_yfwd), big))) return e;
    if ((e = smem_opt_in(reinterpret_cast<const void*>(kb_yinv), big))) return e;
    if ((e = smem_opt_in(reinterpret_cast<const void*>(kb_xconv), big))) return e;
    return smem_opt_in(reinterpret_cast<const void*>(kb_zinv), big);
}

// blocks: the five passes' block counts (z, y, x forward; y, z inverse)
cudaError_t launch_batch_convolve(const BatchBeam* beams, const int* sz, const int* sy, const int* sx,
                                  const int* syi, const int* szi, int nb, const int blocks[5], const size_t smem[3],
                                  cudaStream_t s, int part) {
    if (nb <= 0) return cudaSuccess;
    if (part != CONV_REST) {
        launch(kb_zfwd, blocks[0], FFT_THREADS, smem[0], s, beams, sz, nb);
        launch(kb_yfwd, blocks[1], FFT_THREADS, smem[1], s, beams, sy, nb);
    }
    if (part == CONV_FORWARD) return cudaGetLastError();
    launch(kb_xconv, blocks[2], FFT_THREADS, smem[2], s, beams, sx, nb);
    launch(kb_yinv, blocks[3], FFT_THREADS, smem[1], s, beams, syi, nb);
    launch(kb_zinv, blocks[4], FFT_THREADS, smem[0], s, beams, szi, nb);
    return cudaGetLastError();
}

cudaError_t launch_batch_field(const BatchBeam* beams, const int* start, int nb, int blocks, cudaStream_t s) {
    if (nb <= 0) return cudaSuccess;
    launch(kb_field_octs, blocks, 128, 0, s, beams, start, nb);
    return cudaGetLastError();
}

}  // namespace ocsc
