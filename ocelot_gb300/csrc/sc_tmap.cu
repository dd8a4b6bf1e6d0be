// First-order transport between kicks: X <- R.X + B over the 6 rows of
// rparticles, in place.  Restates TransferMap.mul_p_array
// (ocelot/cpbd/transformations/transfer_map.py:40-50), whose np.dot(R, X)
// is a BLAS product; each output is accumulated as an FMA chain over the six
// inputs in index order and then offset by B.  One thread per particle reads
// its six coordinates (coalesced along each row) and writes six: 96 bytes of
// HBM traffic per particle, nothing else.
#include "sc_common.cuh"

namespace ocsc {

struct Map6 {
    double m[42];  // R (row-major), then B
};

// A map coefficient and whether it is non-zero, tested on its bit pattern:
// on this GPU a double compare issues on the narrow FP64 pipe, an integer
// compare does not.  Every thread reads the same coefficient, so the branch on
// it is warp-uniform.  Skipping a zero term leaves every sum unchanged (up to
// the sign of an exact zero, which the final "+ B" removes) for finite inputs.
// The map may sit in global or shared memory (generic loads).
__device__ __forceinline__ bool coef_nz(const double* m, int i, double& v) {
    const long long b = reinterpret_cast<const long long*>(m)[i];
    v = __longlong_as_double(b);
    return (b << 1) != 0;
}

// y_r = sum_k R[r][k] x_k over the non-zero R[r][k], in k order (FMA chain)
__device__ __forceinline__ void rmul_sparse(const double* m, const double (&x)[6], double (&y)[6]) {
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            double v;
            if (coef_nz(m, r * 6 + k, v)) acc = __fma_rn(v, x[k], acc);
        }
        y[r] = acc;
    }
}

// R entries of an untilted drift/quadrupole map: the 2x2 x and y blocks, R44, R45, R55
constexpr unsigned long long R_PLANAR = (1ull << 0) | (1ull << 1) | (1ull << 6) | (1ull << 7) | (1ull << 14) |
                                        (1ull << 15) | (1ull << 20) | (1ull << 21) | (1ull << 28) | (1ull << 29) |
                                        (1ull << 35);

// whether every non-zero R entry of the map lies in R_PLANAR (one thread, once per block)
__device__ __forceinline__ bool r_is_planar(const double* m) {
    long long any = 0;
    for (int i = 0; i < 36; ++i)
        if (!((R_PLANAR >> i) & 1ull)) any |= reinterpret_cast<const long long*>(m)[i] << 1;
    return any == 0;
}

// one particle: x <- R.x + B with m = R (row-major) then B; planar: R lies in
// R_PLANAR, so only those entries are read (the same FMAs in the same order
// as rmul_sparse over the non-zero entries)
__device__ __forceinline__ void tmap_one(const double* m, double* __restrict__ rp, int64_t ld, int64_t i,
                                         bool planar) {
    double x[6], y[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) x[k] = rp[k * ld + i];
    if (planar) {
        y[0] = __fma_rn(m[1], x[1], __fma_rn(m[0], x[0], 0.0));
        y[1] = __fma_rn(m[7], x[1], __fma_rn(m[6], x[0], 0.0));
        y[2] = __fma_rn(m[15], x[3], __fma_rn(m[14], x[2], 0.0));
        y[3] = __fma_rn(m[21], x[3], __fma_rn(m[20], x[2], 0.0));
        y[4] = __fma_rn(m[29], x[5], __fma_rn(m[28], x[4], 0.0));
        y[5] = __fma_rn(m[35], x[5], 0.0);
    } else {
        rmul_sparse(m, x, y);
    }
    // + B, skipping the zero offsets (the usual case): y + 0 is y
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double b;
        rp[r * ld + i] = coef_nz(m, 36 + r, b) ? __dadd_rn(y[r], b) : y[r];
    }
}

__global__ void __launch_bounds__(256) k_tmap(Map6 m, double* __restrict__ rp, int64_t ld, int64_t n) {
    pdl_wait();
    __shared__ double sm[42];
    __shared__ bool planar;
    if (threadIdx.x < 42) sm[threadIdx.x] = m.m[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) planar = r_is_planar(sm);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        tmap_one(sm, rp, ld, i, planar);
}

// batched: each beam's own map from the work table, over the beam's blocks
__global__ void __launch_bounds__(256) kb_tmap(const BatchBeam* __restrict__ beams, const int* __restrict__ start,
                                               int nb) {
    pdl_wait();
    __shared__ double m[42];
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    if (!B.has_tm) return;
    const VBlk vb = batch_vblk(start, b, B.gx[BS_TMAP], 1);
    __shared__ bool planar;
    if (threadIdx.x < 42) m[threadIdx.x] = B.tm[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) planar = r_is_planar(m);
    __syncthreads();
    const int64_t n = B.kp.n, ld = B.kp.ld;
    for (int64_t i = vb.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)vb.nx * blockDim.x)
        tmap_one(m, B.rp, ld, i, planar);
}

cudaError_t launch_batch_tmap(const BatchBeam* beams, const int* start, int nb, int blocks, cudaStream_t s) {
    if (nb <= 0 || blocks <= 0) return cudaSuccess;
    launch(kb_tmap, blocks, 256, 0, s, beams, start, nb);
    return cudaGetLastError();
}

// Map i = *counter of a device table of maps (row-major R[36] then B[6] per
// map): the transport step of a device-resident tracking loop whose launches
// are recorded once (a CUDA graph) and replayed step after step.  Every block
// reads the counter before k_advance (the next launch on the stream) moves it.
__global__ void __launch_bounds__(256) k_tmap_indexed(const double* __restrict__ table, const int* __restrict__ counter,
                                                      int nmaps, double* __restrict__ rp, int64_t ld, int64_t n) {
    pdl_wait();
    __shared__ double m[42];
    const int idx = *counter;
    if (idx < 0 || idx >= nmaps) return;
    __shared__ bool planar;
    if (threadIdx.x < 42) m[threadIdx.x] = table[(size_t)idx * 42 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) planar = r_is_planar(m);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        tmap_one(m, rp, ld, i, planar);
}

__global__ void k_advance(int* counter, int delta) {
    pdl_wait(); *counter += delta; }

cudaError_t launch_tmap_indexed(const double* table, int* counter, int nmaps, double* rp, int64_t ld, int64_t n,
                                cudaStream_t s) {
    if (n <= 0) {
        launch(k_advance, 1, 1, 0, s, counter, 1);
        return cudaGetLastError();
    }
    int dev = 0, sm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    int64_t b = (n + 255) / 256;
    const int64_t cap = (int64_t)sm * 8;
    if (b > cap) b = cap;
    launch(k_tmap_indexed, (int)b, 256, 0, s, table, counter, nmaps, rp, ld, n);
    launch(k_advance, 1, 1, 0, s, counter, 1);
    return cudaGetLastError();
}

cudaError_t launch_tmap(const double* R, const double* B, double* rp, int64_t ld, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    Map6 m;
    for (int i = 0; i < 36; ++i) m.m[i] = R[i];
    for (int i = 0; i < 6; ++i) m.m[36 + i] = B[i];
    int dev = 0, sm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    int64_t b = (n + 255) / 256;
    const int64_t cap = (int64_t)sm * 8;
    if (b > cap) b = cap;
    launch(k_tmap, (int)b, 256, 0, s, m, rp, ld, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Second-order maps (SecondTM of drift/quadrupole slices,
// ocelot/cpbd/transformations/second_order.py:31-38):
//   y = R.x + sum_{j<=k} Tc[i][jk] x_j x_k,   x <- y + B
// with Tc the combined coefficient T[i,j,k] + T[i,k,j] (j < k) or T[i,j,j].
// A map is MAP2 doubles: R (row-major), B, then Tc[6][21] with the pairs
// (j, k), j <= k, in lexicographic order.  Every thread reads the same map
// entries, so the tests that skip a zero coefficient (coef_nz) are warp-uniform.
// ---------------------------------------------------------------------------
constexpr int MAP2 = 36 + 6 + 6 * 21;

__device__ __forceinline__ void tmap2_one(const double* __restrict__ m, double (&x)[6]) {
    double y[6];
    rmul_sparse(m, x, y);
    // the second-order terms pair by pair: a product x_j x_k is formed only
    // when some output uses it; each output still takes its terms in pair order
    int q = 0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
        for (int k = j; k < 6; ++k, ++q) {
            long long any = 0;
#pragma unroll
            for (int r = 0; r < 6; ++r) any |= reinterpret_cast<const long long*>(m)[42 + r * 21 + q] << 1;
            if (any == 0) continue;
            const double p = __dmul_rn(x[j], x[k]);
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                double v;
                if (coef_nz(m, 42 + r * 21 + q, v)) y[r] = __fma_rn(v, p, y[r]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) x[r] = __dadd_rn(y[r], __ldg(m + 36 + r));
}

// Maps of untilted drifts and quadrupoles without offsets (SC_SLICE_MAP_PLANAR,
// SC_SLICE_MAP_DRIFT): their non-zero R and Tc entries lie in a fixed pattern
// -- R in the 2x2 x and y blocks, R44, R45, R55; Tc in the chromatic terms of
// x, px, y, py and the path-length terms of tau -- which the host checks
// before it marks a record so.  The same FMAs as tmap2_one in the same order
// per output, over the pattern only: no coefficient tests, 11 (drift: 5)
// products instead of up to 21.
__device__ __forceinline__ double mr(const double* __restrict__ m, int r, int k) { return __ldg(m + r * 6 + k); }
__device__ __forceinline__ double mt(const double* __restrict__ m, int r, int q) { return __ldg(m + 42 + r * 21 + q); }

__device__ __forceinline__ void add_b(const double* __restrict__ m, double (&y)[6], double (&x)[6]) {
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double b;
        x[r] = coef_nz(m, 36 + r, b) ? __dadd_rn(y[r], b) : y[r];
    }
}

__device__ __forceinline__ void planar_one(const double* __restrict__ m, double (&x)[6]) {
    const double p00 = __dmul_rn(x[0], x[0]), p01 = __dmul_rn(x[0], x[1]), p05 = __dmul_rn(x[0], x[5]);
    const double p11 = __dmul_rn(x[1], x[1]), p15 = __dmul_rn(x[1], x[5]), p22 = __dmul_rn(x[2], x[2]);
    const double p23 = __dmul_rn(x[2], x[3]), p25 = __dmul_rn(x[2], x[5]), p33 = __dmul_rn(x[3], x[3]);
    const double p35 = __dmul_rn(x[3], x[5]), p55 = __dmul_rn(x[5], x[5]);
    double y[6];
    y[0] = __fma_rn(mr(m, 0, 1), x[1], __fma_rn(mr(m, 0, 0), x[0], 0.0));
    y[0] = __fma_rn(mt(m, 0, 10), p15, __fma_rn(mt(m, 0, 5), p05, y[0]));
    y[1] = __fma_rn(mr(m, 1, 1), x[1], __fma_rn(mr(m, 1, 0), x[0], 0.0));
    y[1] = __fma_rn(mt(m, 1, 10), p15, __fma_rn(mt(m, 1, 5), p05, y[1]));
    y[2] = __fma_rn(mr(m, 2, 3), x[3], __fma_rn(mr(m, 2, 2), x[2], 0.0));
    y[2] = __fma_rn(mt(m, 2, 17), p35, __fma_rn(mt(m, 2, 14), p25, y[2]));
    y[3] = __fma_rn(mr(m, 3, 3), x[3], __fma_rn(mr(m, 3, 2), x[2], 0.0));
    y[3] = __fma_rn(mt(m, 3, 17), p35, __fma_rn(mt(m, 3, 14), p25, y[3]));
    double a = __fma_rn(mr(m, 4, 5), x[5], __fma_rn(mr(m, 4, 4), x[4], 0.0));
    a = __fma_rn(mt(m, 4, 6), p11, __fma_rn(mt(m, 4, 1), p01, __fma_rn(mt(m, 4, 0), p00, a)));
    a = __fma_rn(mt(m, 4, 15), p33, __fma_rn(mt(m, 4, 12), p23, __fma_rn(mt(m, 4, 11), p22, a)));
    y[4] = __fma_rn(mt(m, 4, 20), p55, a);
    y[5] = __fma_rn(mr(m, 5, 5), x[5], 0.0);
    add_b(m, y, x);
}

__device__ __forceinline__ void drift_one(const double* __restrict__ m, double (&x)[6]) {
    const double p11 = __dmul_rn(x[1], x[1]), p15 = __dmul_rn(x[1], x[5]), p33 = __dmul_rn(x[3], x[3]);
    const double p35 = __dmul_rn(x[3], x[5]), p55 = __dmul_rn(x[5], x[5]);
    double y[6];
    y[0] = __fma_rn(mt(m, 0, 10), p15, __fma_rn(mr(m, 0, 1), x[1], __fma_rn(mr(m, 0, 0), x[0], 0.0)));
    y[1] = __fma_rn(mr(m, 1, 1), x[1], 0.0);
    y[2] = __fma_rn(mt(m, 2, 17), p35, __fma_rn(mr(m, 2, 3), x[3], __fma_rn(mr(m, 2, 2), x[2], 0.0)));
    y[3] = __fma_rn(mr(m, 3, 3), x[3], 0.0);
    double a = __fma_rn(mr(m, 4, 5), x[5], __fma_rn(mr(m, 4, 4), x[4], 0.0));
    y[4] = __fma_rn(mt(m, 4, 20), p55, __fma_rn(mt(m, 4, 15), p33, __fma_rn(mt(m, 4, 6), p11, a)));
    y[5] = __fma_rn(mr(m, 5, 5), x[5], 0.0);
    add_b(m, y, x);
}

// first-order maps (Tc = 0) in the R pattern of planar_one (SC_SLICE_MAP_LINEAR)
__device__ __forceinline__ void linear_one(const double* __restrict__ m, double (&x)[6]) {
    double y[6];
    y[0] = __fma_rn(mr(m, 0, 1), x[1], __fma_rn(mr(m, 0, 0), x[0], 0.0));
    y[1] = __fma_rn(mr(m, 1, 1), x[1], __fma_rn(mr(m, 1, 0), x[0], 0.0));
    y[2] = __fma_rn(mr(m, 2, 3), x[3], __fma_rn(mr(m, 2, 2), x[2], 0.0));
    y[3] = __fma_rn(mr(m, 3, 3), x[3], __fma_rn(mr(m, 3, 2), x[2], 0.0));
    y[4] = __fma_rn(mr(m, 4, 5), x[5], __fma_rn(mr(m, 4, 4), x[4], 0.0));
    y[5] = __fma_rn(mr(m, 5, 5), x[5], 0.0);
    add_b(m, y, x);
}

// An RF cavity slice, CavityTM.map4cav (ocelot/cpbd/transformations/cavity.py:29-128):
// the first-order map x <- R.x + B of the slice, then, from the coordinates
// before it,
//   x5 <- x5_0 E beta0 / (E1 beta1) + V beta0 / (E1 beta1) (cos(-x4_0 beta0 k + phi) - cos phi)
//   x4 <- x4 + T566 x5_0^2 + T556 x4_0 x5_0 + T555 x4_0^2
// with the reference's operation order (the products left to right, one
// division).  A cavity record is MAP2 doubles: R, B, then the slice's scalars
// at CAV_*; when the energy after the slice is not positive only the T566
// term is applied and x5 keeps its first-order value (cavity.py:67-70).
constexpr int CAV_E = 42, CAV_BETA0 = 43, CAV_DEN = 44, CAV_A = 45, CAV_K = 46, CAV_PHI = 47, CAV_COSPHI = 48,
              CAV_T566 = 49, CAV_T556 = 50, CAV_T555 = 51, CAV_RF = 52, CAV_RDEN = 53, CAV_SINPHI = 54,
              CAV_RPAT = 55;

// cos(arg) for arg = phi + d with |d| <= 1/4: cos(phi) + (cos(phi) (cos d - 1) - sin(phi) sin d), the two
// series in d^2 (Taylor, to d^16 and d^15: truncation below 1e-22 of the result) by Horner's rule
__device__ __forceinline__ double cos_near(double d, double cphi, double sphi) {
    const double z = __dmul_rn(d, d);
    double c = __fma_rn(z, -1.0 / 20922789888000.0, 1.0 / 87178291200.0);
    c = __fma_rn(z, c, -1.0 / 479001600.0);
    c = __fma_rn(z, c, 1.0 / 3628800.0);
    c = __fma_rn(z, c, -1.0 / 40320.0);
    c = __fma_rn(z, c, 1.0 / 720.0);
    c = __fma_rn(z, c, -1.0 / 24.0);
    c = __fma_rn(z, c, 0.5);
    const double cm1 = -__dmul_rn(z, c);            // cos d - 1
    double s = __fma_rn(z, -1.0 / 1307674368000.0, 1.0 / 6227020800.0);
    s = __fma_rn(z, s, -1.0 / 39916800.0);
    s = __fma_rn(z, s, 1.0 / 362880.0);
    s = __fma_rn(z, s, -1.0 / 5040.0);
    s = __fma_rn(z, s, 1.0 / 120.0);
    s = __fma_rn(z, s, -1.0 / 6.0);
    const double sd = __fma_rn(__dmul_rn(z, d), s, d);   // sin d
    return __dadd_rn(cphi, __fma_rn(cphi, cm1, -__dmul_rn(sphi, sd)));
}

__device__ __forceinline__ void cavity_one(const double* __restrict__ m, double (&x)[6]) {
    const double x4 = x[4], x5 = x[5];
    // R: when the host found it in the pattern of cavity_R_z (x and y blocks, longitudinal 2x2 block; untilted),
    // those 12 entries in k order per output, else the general sparse product -- the same FMAs either way
    double y[6];
    if (__ldg(reinterpret_cast<const long long*>(m) + CAV_RPAT) != 0) {
        y[0] = __fma_rn(mr(m, 0, 1), x[1], __fma_rn(mr(m, 0, 0), x[0], 0.0));
        y[1] = __fma_rn(mr(m, 1, 1), x[1], __fma_rn(mr(m, 1, 0), x[0], 0.0));
        y[2] = __fma_rn(mr(m, 2, 3), x[3], __fma_rn(mr(m, 2, 2), x[2], 0.0));
        y[3] = __fma_rn(mr(m, 3, 3), x[3], __fma_rn(mr(m, 3, 2), x[2], 0.0));
        y[4] = __fma_rn(mr(m, 4, 5), x[5], __fma_rn(mr(m, 4, 4), x[4], 0.0));
        y[5] = __fma_rn(mr(m, 5, 5), x[5], __fma_rn(mr(m, 5, 4), x[4], 0.0));
    } else {
        rmul_sparse(m, x, y);
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double b;
        if (coef_nz(m, 36 + r, b)) y[r] = __dadd_rn(y[r], b);
    }
    const double t566 = __ldg(m + CAV_T566);
    if (__ldg(m + CAV_RF) != 0.0) {
        const double beta0 = __ldg(m + CAV_BETA0);
        // a / D by a product with y = RN(1/D) and one correction, q + (a - qD) y (Markstein's division)
        const double a = __dmul_rn(__dmul_rn(x5, __ldg(m + CAV_E)), beta0);
        const double den = __ldg(m + CAV_DEN), rden = __ldg(m + CAV_RDEN);
        const double q = __dmul_rn(a, rden);
        const double lin = __fma_rn(__fma_rn(-q, den, a), rden, q);
        const double phi = __ldg(m + CAV_PHI), cphi = __ldg(m + CAV_COSPHI);
        const double arg = __dadd_rn(__dmul_rn(__dmul_rn(-x4, beta0), __ldg(m + CAV_K)), phi);
        const double d = __dsub_rn(arg, phi);
        const double c = fabs(d) <= 0.25 ? cos_near(d, cphi, __ldg(m + CAV_SINPHI)) : cos(arg);
        y[5] = __dadd_rn(lin, __dmul_rn(__ldg(m + CAV_A), __dsub_rn(c, cphi)));
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(t566, x5), x5),
                                             __dmul_rn(__dmul_rn(__ldg(m + CAV_T556), x4), x5)),
                                   __dmul_rn(__dmul_rn(__ldg(m + CAV_T555), x4), x4));
        y[4] = __dadd_rn(y[4], s);
    } else {
        y[4] = __dadd_rn(y[4], __dmul_rn(__dmul_rn(t566, x5), x5));
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) x[r] = y[r];
}

// maps [first, last) of the table applied in order to every particle, its
// coordinates kept in registers between maps; kinds (optional) marks the
// cavity slices and the maps of the fixed drift/quadrupole patterns, the
// others are general second-order maps
__device__ __forceinline__ void tmap2_range(const double* __restrict__ maps, const int* __restrict__ kinds, int first,
                                            int last, double* __restrict__ rp, int64_t ld, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = rp[k * ld + i];
        for (int mi = first; mi < last; ++mi) {
            const int kind = kinds != nullptr ? __ldg(kinds + mi) : SC_SLICE_MAP;
            const double* m = maps + (size_t)mi * MAP2;
            if (kind == SC_SLICE_MAP_DRIFT)
                drift_one(m, x);
            else if (kind == SC_SLICE_MAP_LINEAR)
                linear_one(m, x);
            else if (kind == SC_SLICE_MAP_PLANAR)
                planar_one(m, x);
            else if (kind == SC_SLICE_CAVITY)
                cavity_one(m, x);
            else
                tmap2_one(m, x);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) rp[k * ld + i] = x[k];
    }
}

__global__ void __launch_bounds__(256) k_tmap2(const double* __restrict__ maps, const int* __restrict__ kinds,
                                               int nmaps, double* __restrict__ rp, int64_t ld, int64_t n) {
    pdl_wait();
    tmap2_range(maps, kinds, 0, nmaps, rp, ld, n);
}

// the maps of step *counter: [first[*counter], first[*counter + 1]) (a
// device-resident tracking loop's transport, replayed from a CUDA graph)
__global__ void __launch_bounds__(256) k_tmap2_step(const double* __restrict__ maps, const int* __restrict__ kinds,
                                                    const int* __restrict__ first, const int* __restrict__ counter,
                                                    int nsteps, double* __restrict__ rp, int64_t ld, int64_t n) {
    pdl_wait();
    const int step = *counter;
    if (step < 0 || step >= nsteps) return;
    tmap2_range(maps, kinds, first[step], first[step + 1], rp, ld, n);
}

static int tmap_blocks(int64_t n) {
    int dev = 0, sm = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    int64_t b = (n + 255) / 256;
    const int64_t cap = (int64_t)sm * 8;
    if (b > cap) b = cap;
    return (int)(b > 0 ? b : 1);
}

cudaError_t launch_tmap2(const double* maps, const int* kinds, int nmaps, double* rp, int64_t ld, int64_t n,
                         cudaStream_t s) {
    if (n <= 0 || nmaps <= 0) return cudaSuccess;
    launch(k_tmap2, tmap_blocks(n), 256, 0, s, maps, kinds, nmaps, rp, ld, n);
    return cudaGetLastError();
}

cudaError_t launch_tmap2_step(const double* maps, const int* kinds, const int* first, int* counter, int nsteps,
                              double* rp, int64_t ld, int64_t n, cudaStream_t s) {
    if (n > 0) launch(k_tmap2_step, tmap_blocks(n), 256, 0, s, maps, kinds, first, counter, nsteps, rp, ld, n);
    launch(k_advance, 1, 1, 0, s, counter, 1);
    return cudaGetLastError();
}

}  // namespace ocsc

namespace ocsc {

// ---------------------------------------------------------------------------
// Beam moments of get_envelope (ocelot/cpbd/beam/analysis.py:27-226) without
// dispersion correction: the means of x, y, px', py', tau, p and the twelve
// central second moments, with px' = px f, py' = py f,
// f = 1 - p - p^2/2 + px^2/2 + py^2/2, over all particles or over those with
// tau within [m + lo s, m + hi s] (m, s: mean and standard deviation of tau).
// One pass over the rows (two with bounds: the tau statistics first): the
// sums of d = v - v0 and of the products d_v d_w, shifted by the first
// particle's values v0, give mean = v0 + S1/n and central moment
// S2/n - (S1/n)(S1/n) -- the shift keeps the subtraction free of
// cancellation for any beam offset.  Each pass is one launch: every block
// reduces its grid-stride share and writes its partial sums, and the last
// block to finish (a ticket) adds the partials in block order -- so the sums
// are deterministic -- and writes the slot *counter of the output table.
// ---------------------------------------------------------------------------
constexpr int MOM_BLOCKS = 304, MOM_THREADS = 256, MOM_K = 19;

__device__ __forceinline__ void mom_prime(const double* __restrict__ X, int64_t ld, int64_t i, double (&v)[6]) {
    // x, y, px', py', tau, p of particle i (the factor with get_envelope's operations, as FMAs)
    const double px = X[ld + i], py = X[3 * ld + i], p = X[5 * ld + i];
    double f = __fma_rn(-__dmul_rn(0.5, p), p, __dsub_rn(1.0, p));
    f = __fma_rn(__dmul_rn(0.5, px), px, f);
    f = __fma_rn(__dmul_rn(0.5, py), py, f);
    v[0] = X[i];
    v[1] = X[2 * ld + i];
    v[2] = __dmul_rn(px, f);
    v[3] = __dmul_rn(py, f);
    v[4] = X[4 * ld + i];
    v[5] = p;
}

__global__ void __launch_bounds__(MOM_THREADS) k_moments(const double* __restrict__ rp, int64_t ld, int64_t n,
                                                        const int* __restrict__ counter, int nslots, int pass,
                                                        int use_bounds, double lo, double hi, double* out,
                                                        double* __restrict__ partial, unsigned int* ticket) {
    pdl_wait();
    const int slot = counter ? *counter : 0;
    if (slot < 0 || slot >= nslots) return;
    double* o = out + (size_t)slot * SC_MOMENTS;
    double acc[MOM_K];
#pragma unroll
    for (int k = 0; k < MOM_K; ++k) acc[k] = 0.0;
    double v0[6];
    mom_prime(rp, ld, 0, v0);
    double tlo = -INFINITY, thi = INFINITY;
    if (pass == 1 && use_bounds) {
        tlo = __dadd_rn(o[1], __dmul_rn(o[2], lo));
        thi = __dadd_rn(o[1], __dmul_rn(o[2], hi));
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double tau = rp[4 * ld + i];
        if (pass == 0) {
            const double d = __dsub_rn(tau, v0[4]);
            acc[0] += d;
            acc[1] = __fma_rn(d, d, acc[1]);
            continue;
        }
        if (!(tlo <= tau && tau <= thi)) continue;
        double v[6];
        mom_prime(rp, ld, i, v);
        double d[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) d[k] = __dsub_rn(v[k], v0[k]);
        acc[0] += 1.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[1 + k] += d[k];
        // xx, xpx, pxpx, yy, ypy, pypy, tautau, xy, pxpy, xpy, ypx, pp (d: x, y, px, py, tau, p)
        acc[7] = __fma_rn(d[0], d[0], acc[7]);    acc[8] = __fma_rn(d[0], d[2], acc[8]);
        acc[9] = __fma_rn(d[2], d[2], acc[9]);    acc[10] = __fma_rn(d[1], d[1], acc[10]);
        acc[11] = __fma_rn(d[1], d[3], acc[11]);  acc[12] = __fma_rn(d[3], d[3], acc[12]);
        acc[13] = __fma_rn(d[4], d[4], acc[13]);  acc[14] = __fma_rn(d[0], d[1], acc[14]);
        acc[15] = __fma_rn(d[2], d[3], acc[15]);  acc[16] = __fma_rn(d[0], d[3], acc[16]);
        acc[17] = __fma_rn(d[1], d[2], acc[17]);  acc[18] = __fma_rn(d[5], d[5], acc[18]);
    }
    const int nk = pass == 0 ? 2 : MOM_K;
    __shared__ double s_red[MOM_THREADS / 32][MOM_K];
    __shared__ double s_sum[MOM_K];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < MOM_K; ++k) {
        if (k >= nk) break;
        double v = acc[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) s_red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < nk) {
        double v = 0.0;
        for (int w = 0; w < MOM_THREADS / 32; ++w) v += s_red[w][threadIdx.x];
        partial[(size_t)blockIdx.x * MOM_K + threadIdx.x] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (threadIdx.x < nk) {
        double v = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) v += __ldcg(partial + (size_t)b * MOM_K + threadIdx.x);
        s_sum[threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (pass == 0) {
            const double m1 = s_sum[0] / (double)n;
            o[1] = __dadd_rn(v0[4], m1);
            o[2] = sqrt(fmax(__fma_rn(-m1, m1, s_sum[1] / (double)n), 0.0));
        } else {
            const double cnt = s_sum[0];
            o[0] = cnt;
            double m1[6];
            for (int k = 0; k < 6; ++k) {
                m1[k] = s_sum[1 + k] / cnt;
                o[3 + k] = __dadd_rn(v0[k], m1[k]);
            }
            const int a[12] = {0, 0, 2, 1, 1, 3, 4, 0, 2, 0, 1, 5};
            const int b[12] = {0, 2, 2, 1, 3, 3, 4, 1, 3, 3, 2, 5};
            for (int k = 0; k < 12; ++k) {
                double c = __fma_rn(-m1[a[k]], m1[b[k]], s_sum[7 + k] / cnt);
                if (a[k] == b[k]) c = fmax(c, 0.0);   // a variance: not below 0 by rounding
                o[9 + k] = cnt == 1.0 ? 0.0 : c;      // one particle: no spread, exactly
            }
        }
        *ticket = 0u;
    }
}

cudaError_t launch_moments(const double* rp, int64_t ld, int64_t n, const int* counter, int nslots, int use_bounds,
                           double lo, double hi, double* out, void* scratch, cudaStream_t s) {
    double* partial = (double*)scratch;
    unsigned int* ticket = (unsigned int*)(partial + (size_t)MOM_BLOCKS * MOM_K);
    int64_t b = (n + MOM_THREADS - 1) / MOM_THREADS;
    const int blocks = (int)(b < 1 ? 1 : (b > MOM_BLOCKS ? MOM_BLOCKS : b));
    for (int pass = use_bounds ? 0 : 1; pass < 2; ++pass)
        launch(k_moments, blocks, MOM_THREADS, 0, s, rp, ld, n, counter, nslots, pass, use_bounds, lo, hi, out,
               partial, ticket);
    return cudaGetLastError();
}

size_t moments_scratch_bytes() { return (size_t)MOM_BLOCKS * MOM_K * sizeof(double) + 64; }

}  // namespace ocsc
