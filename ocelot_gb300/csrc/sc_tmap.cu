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

// one particle: x <- R.x + B with m = R (row-major) then B
__device__ __forceinline__ void tmap_one(const double* __restrict__ m, double* __restrict__ rp, int64_t ld,
                                         int64_t i) {
    double x[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) x[k] = rp[k * ld + i];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double acc = __dmul_rn(m[r * 6], x[0]);
#pragma unroll
        for (int k = 1; k < 6; ++k) acc = __fma_rn(m[r * 6 + k], x[k], acc);
        rp[r * ld + i] = __dadd_rn(acc, m[36 + r]);
    }
}

__global__ void __launch_bounds__(256) k_tmap(Map6 m, double* __restrict__ rp, int64_t ld, int64_t n) {
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        tmap_one(m.m, rp, ld, i);
}

// batched: each beam's own map from the work table, over the beam's blocks
__global__ void __launch_bounds__(256) kb_tmap(const BatchBeam* __restrict__ beams, const int* __restrict__ start,
                                               int nb) {
    pdl_wait();
    __shared__ double m[42];
    const int b = batch_beam(start, nb);
    const BatchBeam& B = beams[b];
    if (!B.has_tm) return;
    const VBlk vb = batch_vblk(start, b, B.gx[BS_PART], 1);
    if (threadIdx.x < 42) m[threadIdx.x] = B.tm[threadIdx.x];
    __syncthreads();
    const int64_t n = B.kp.n, ld = B.kp.ld;
    for (int64_t i = vb.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)vb.nx * blockDim.x)
        tmap_one(m, B.rp, ld, i);
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
    if (threadIdx.x < 42) m[threadIdx.x] = table[(size_t)idx * 42 + threadIdx.x];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        tmap_one(m, rp, ld, i);
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
// entries, so the test that skips a zero coefficient is warp-uniform.
// ---------------------------------------------------------------------------
constexpr int MAP2 = 36 + 6 + 6 * 21;

__device__ __forceinline__ void tmap2_one(const double* __restrict__ m, double (&x)[6]) {
    double p[21];
    int q = 0;
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
        for (int k = j; k < 6; ++k) p[q++] = __dmul_rn(x[j], x[k]);
    double y[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double acc = __dmul_rn(__ldg(m + r * 6), x[0]);
#pragma unroll
        for (int k = 1; k < 6; ++k) acc = __fma_rn(__ldg(m + r * 6 + k), x[k], acc);
#pragma unroll
        for (int t = 0; t < 21; ++t) {
            const double v = __ldg(m + 42 + r * 21 + t);
            if (v != 0.0) acc = __fma_rn(v, p[t], acc);
        }
        y[r] = acc;
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) x[r] = __dadd_rn(y[r], __ldg(m + 36 + r));
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
              CAV_T566 = 49, CAV_T556 = 50, CAV_T555 = 51, CAV_RF = 52;

__device__ __forceinline__ void cavity_one(const double* __restrict__ m, double (&x)[6]) {
    const double x4 = x[4], x5 = x[5];
    double y[6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double acc = __dmul_rn(__ldg(m + r * 6), x[0]);
#pragma unroll
        for (int k = 1; k < 6; ++k) acc = __fma_rn(__ldg(m + r * 6 + k), x[k], acc);
        y[r] = __dadd_rn(acc, __ldg(m + 36 + r));
    }
    const double t566 = __ldg(m + CAV_T566);
    if (__ldg(m + CAV_RF) != 0.0) {
        const double beta0 = __ldg(m + CAV_BETA0);
        const double lin = __ddiv_rn(__dmul_rn(__dmul_rn(x5, __ldg(m + CAV_E)), beta0), __ldg(m + CAV_DEN));
        const double arg = __dadd_rn(__dmul_rn(__dmul_rn(-x4, beta0), __ldg(m + CAV_K)), __ldg(m + CAV_PHI));
        y[5] = __dadd_rn(lin, __dmul_rn(__ldg(m + CAV_A), __dsub_rn(cos(arg), __ldg(m + CAV_COSPHI))));
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
// cavity slices (SC_SLICE_CAVITY), the others are second-order maps
__device__ __forceinline__ void tmap2_range(const double* __restrict__ maps, const int* __restrict__ kinds, int first,
                                            int last, double* __restrict__ rp, int64_t ld, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = rp[k * ld + i];
        for (int mi = first; mi < last; ++mi) {
            if (kinds != nullptr && __ldg(kinds + mi) == SC_SLICE_CAVITY)
                cavity_one(maps + (size_t)mi * MAP2, x);
            else
                tmap2_one(maps + (size_t)mi * MAP2, x);
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
