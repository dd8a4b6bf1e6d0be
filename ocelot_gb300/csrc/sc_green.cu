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
#include "sc_common.cuh"
#include "sc_fft_dev.cuh"

namespace ocsc {

struct IgfArgs {
    double hx, hy, hz;
    int use_state;  // take the spacing from ScState::steps
    int force;      // build even if the cache is valid
};

__device__ __forceinline__ bool igf_skip(const ScState* st, const IgfArgs& a) {
    if (a.force) return false;
    return st->status != SC_OK || !st->igf_rebuild;
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

__global__ void k_igf_corners(double* __restrict__ ig, int nx, int ny, int nz, IgfArgs a, const ScState* st) {
    if (igf_skip(st, a)) return;
    double hx = a.hx, hy = a.hy, hz = a.hz;
    if (a.use_state) { hx = st->steps[0]; hy = st->steps[1]; hz = st->steps[2]; }
    const int cx1 = nx + 1, cy1 = ny + 1, cz1 = nz + 1;
    const size_t total = (size_t)cx1 * cy1 * cz1;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < total; c += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(c % cz1);
        const int j = (int)((c / cz1) % cy1);
        const int i = (int)(c / ((size_t)cz1 * cy1));
        const double x = __dsub_rn(__dmul_rn(hx, (double)i), __dmul_rn(hx, 0.5));
        const double y = __dsub_rn(__dmul_rn(hy, (double)j), __dmul_rn(hy, 0.5));
        const double z = __dsub_rn(__dmul_rn(hz, (double)k), __dmul_rn(hz, 0.5));
        ig[c] = igf_point(x, y, z);
    }
}

__global__ void k_igf_diff(const double* __restrict__ ig, double* __restrict__ k1, int nx, int ny, int nz,
                           IgfArgs a, const ScState* st) {
    if (igf_skip(st, a)) return;
    const size_t total = (size_t)nx * ny * nz;
    const size_t sy = nz + 1, sx = (size_t)(ny + 1) * (nz + 1);
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < total; c += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(c % nz);
        const int j = (int)((c / nz) % ny);
        const int i = (int)(c / ((size_t)nz * ny));
        const size_t o = i * sx + j * sy + k;
        double v = __dsub_rn(ig[o + sx + sy + 1], ig[o + sy + 1]);
        v = __dsub_rn(v, ig[o + sx + 1]);
        v = __dadd_rn(v, ig[o + 1]);
        v = __dsub_rn(v, ig[o + sx + sy]);
        v = __dadd_rn(v, ig[o + sy]);
        v = __dadd_rn(v, ig[o + sx]);
        v = __dsub_rn(v, ig[o]);
        k1[c] = v;
    }
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
    while (tk > 2 && sizeof(Cx<R>) * (size_t)(M + 2 * tk * (M + 1)) > 200 * 1024) tk /= 2;
    return tk;
}

// S1: along z; rows (x, y) of K1 -> S1[x][y][kz], kz <= Mz/2
template <typename R>
__global__ void __launch_bounds__(GT) k_green_z(const double* __restrict__ k1, R* __restrict__ s1, int ny, int nz,
                                                int Kz, RadixPlan rz, const Cx<R>* __restrict__ twg, int NC,
                                                IgfArgs a, const ScState* st) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (igf_skip(st, a)) return;
    const int Mz = rz.L;
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* A = tw + Mz;
    Cx<R>* B = A + NC * Mz;
    load_twiddles<R>(tw, twg, Mz);
    const int x = blockIdx.y, y0 = blockIdx.x * 2 * NC;
    for (int idx = threadIdx.x; idx < NC * Mz; idx += blockDim.x) {
        const int c = idx / Mz, z = idx - c * Mz;
        const int ya = y0 + 2 * c, yb = ya + 1;
        const int zs = even_src(z, nz, Mz);
        R re = 0, im = 0;
        if (zs >= 0) {
            if (ya < ny) re = (R)k1[((size_t)x * ny + ya) * nz + zs];
            if (yb < ny) im = (R)k1[((size_t)x * ny + yb) * nz + zs];
        }
        A[idx] = cx<R>(re, im);
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, false>(A, B, Mz, NC, rz, tw);
    for (int idx = threadIdx.x; idx < NC * Kz; idx += blockDim.x) {
        const int c = idx / Kz, k = idx - c * Kz;
        const int ya = y0 + 2 * c, yb = ya + 1;
        const Cx<R> v = res[c * Mz + k];
        if (ya < ny) s1[((size_t)x * ny + ya) * Kz + k] = v.x;
        if (yb < ny) s1[((size_t)x * ny + yb) * Kz + k] = v.y;
    }
}

// S2/S3: strided passes over columns kz (paired), line axis of length n -> M,
// input rows in[(o*nin + l)*Kz + kz], output rows out[(o*nout + kl)*Kz + kz]
template <typename R>
__global__ void __launch_bounds__(GT) k_green_strided(const R* __restrict__ in, R* __restrict__ out, int n,
                                                      int nin_stride, int nout, int Kz, int outer_in_stride,
                                                      int outer_out_stride, RadixPlan rp,
                                                      const Cx<R>* __restrict__ twg, int GTK, IgfArgs a,
                                                      const ScState* st) {
    extern __shared__ __align__(16) unsigned char smraw[];
    if (igf_skip(st, a)) return;
    const int M = rp.L, ls = M + 1;
    Cx<R>* tw = reinterpret_cast<Cx<R>*>(smraw);
    Cx<R>* A = tw + M;
    Cx<R>* B = A + GTK * ls;
    load_twiddles<R>(tw, twg, M);
    const int o = blockIdx.y;
    const int k0 = blockIdx.x * 2 * GTK;
    const R* src = in + (size_t)o * outer_in_stride;
    R* dst = out + (size_t)o * outer_out_stride;
    for (int idx = threadIdx.x; idx < M * GTK; idx += blockDim.x) {
        const int l = idx / GTK, kk = idx - l * GTK;
        const int ka = k0 + 2 * kk, kb = ka + 1;
        const int ls_ = even_src(l, n, M);
        R re = 0, im = 0;
        if (ls_ >= 0) {
            if (ka < Kz) re = src[(size_t)ls_ * nin_stride + ka];
            if (kb < Kz) im = src[(size_t)ls_ * nin_stride + kb];
        }
        A[kk * ls + l] = cx<R>(re, im);
    }
    __syncthreads();
    Cx<R>* res = fft_lines<R, false>(A, B, ls, GTK, rp, tw);
    for (int idx = threadIdx.x; idx < nout * GTK; idx += blockDim.x) {
        const int l = idx / GTK, kk = idx - l * GTK;
        const int ka = k0 + 2 * kk, kb = ka + 1;
        const Cx<R> v = res[kk * ls + l];
        if (ka < Kz) dst[(size_t)l * nin_stride + ka] = v.x;
        if (kb < Kz) dst[(size_t)l * nin_stride + kb] = v.y;
    }
}

template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

static int grid_for(size_t work, int sm) {
    size_t b = (work + 255) / 256;
    size_t cap = (size_t)sm * 16;
    return (int)(b < cap ? (b ? b : 1) : cap);
}

static IgfArgs state_args(bool force) {
    IgfArgs a;
    a.hx = a.hy = a.hz = 0;
    a.use_state = 1;
    a.force = force ? 1 : 0;
    return a;
}

cudaError_t launch_igf_h(const Plan& p, const Layout& L, char* ws, double* kern_out, double hx, double hy,
                         double hz, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    IgfArgs a;
    a.hx = hx; a.hy = hy; a.hz = hz;
    a.use_state = 0;
    a.force = 1;
    double* ig = reinterpret_cast<double*>(ws + L.igf_ig);
    const size_t nc = (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
    k_igf_corners<<<grid_for(nc, p.sm_count), 256, 0, s>>>(ig, p.nx, p.ny, p.nz, a, st);
    const size_t nk = (size_t)p.nx * p.ny * p.nz;
    k_igf_diff<<<grid_for(nk, p.sm_count), 256, 0, s>>>(ig, kern_out, p.nx, p.ny, p.nz, a, st);
    return cudaGetLastError();
}

cudaError_t launch_igf(const Plan& p, const Layout& L, char* ws, double* kern_out, bool force, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    IgfArgs a = state_args(force);
    double* ig = reinterpret_cast<double*>(ws + L.igf_ig);
    double* k1 = kern_out ? kern_out : reinterpret_cast<double*>(ws + L.igf_k1);
    const size_t nc = (size_t)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
    k_igf_corners<<<grid_for(nc, p.sm_count), 256, 0, s>>>(ig, p.nx, p.ny, p.nz, a, st);
    const size_t nk = (size_t)p.nx * p.ny * p.nz;
    k_igf_diff<<<grid_for(nk, p.sm_count), 256, 0, s>>>(ig, k1, p.nx, p.ny, p.nz, a, st);
    return cudaGetLastError();
}

template <typename R>
static cudaError_t spectrum_t(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    IgfArgs a = state_args(false);
    const int Kx = p.Mx / 2 + 1, Ky = p.My / 2 + 1, Kz = p.Mz / 2 + 1;
    const double* k1 = reinterpret_cast<const double*>(ws + L.igf_k1);
    R* s1 = reinterpret_cast<R*>(ws + L.green_s1);
    R* s2 = reinterpret_cast<R*>(ws + L.green_s2);
    R* g = reinterpret_cast<R*>(ws + L.green);
    const Cx<R>* twx = reinterpret_cast<const Cx<R>*>(ws + L.tw_x);
    const Cx<R>* twy = reinterpret_cast<const Cx<R>*>(ws + L.tw_y);
    const Cx<R>* twz = reinterpret_cast<const Cx<R>*>(ws + L.tw_z);
    cudaError_t e;
    int NC = 2048 / p.Mz;
    NC = NC < 1 ? 1 : (NC > 16 ? 16 : NC);
    const size_t smz = sizeof(Cx<R>) * (size_t)(p.Mz + 2 * NC * p.Mz);
    if ((e = set_smem(k_green_z<R>, smz))) return e;
    dim3 gz((p.ny + 2 * NC - 1) / (2 * NC), p.nx);
    k_green_z<R><<<gz, GT, smz, s>>>(k1, s1, p.ny, p.nz, Kz, p.rz, twz, NC, a, st);
    // S2 along y: for each x, rows y < ny of S1[x] -> rows ky < Ky of S2[x]
    const int tky = green_cols<R>(p.My), tkx = green_cols<R>(p.Mx);
    const size_t smy = sizeof(Cx<R>) * (size_t)(p.My + 2 * tky * (p.My + 1));
    const size_t smx = sizeof(Cx<R>) * (size_t)(p.Mx + 2 * tkx * (p.Mx + 1));
    if ((e = set_smem(k_green_strided<R>, smx > smy ? smx : smy))) return e;
    dim3 gy((Kz + 2 * tky - 1) / (2 * tky), p.nx);
    k_green_strided<R><<<gy, GT, smy, s>>>(s1, s2, p.ny, Kz, Ky, Kz, p.ny * Kz, Ky * Kz, p.ry, twy, tky, a, st);
    // S3 along x: for each ky, rows x < nx of S2[.][ky] -> rows kx < Kx of G[.][ky]
    dim3 gx((Kz + 2 * tkx - 1) / (2 * tkx), Ky);
    k_green_strided<R><<<gx, GT, smx, s>>>(s2, g, p.nx, Ky * Kz, Kx, Kz, Kz, Kz, p.rx, twx, tkx, a, st);
    return cudaGetLastError();
}

cudaError_t launch_green_spectrum(const Plan& p, const Layout& L, char* ws, cudaStream_t s) {
    return p.prec == SC_FP64 ? spectrum_t<double>(p, L, ws, s) : spectrum_t<float>(p, L, ws, s);
}

}  // namespace ocsc
