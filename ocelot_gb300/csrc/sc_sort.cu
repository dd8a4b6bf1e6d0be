// Deterministic NGP charge deposit: stable radix sort of cell keys followed
// by a segmented sum in particle order.
//
// The reference deposits with np.bincount(inds, Q) (ocelot/cpbd/sc.py:193),
// which adds the charges of each cell sequentially in particle order.  Here
// the keys are sorted by a stable least-significant-digit radix sort
// (ceil(key_bits/9) passes of at most 9-bit digits: two passes for a 64^3
// mesh), which puts the particles of each cell
// in a contiguous run in particle order, the last pass carrying the charges
// themselves; each cell's run is then summed by one warp.  In FP64 the sum is
// a sequential fold and reproduces bincount's sums bit for bit; in FP32 it is
// Kahan-compensated.  The result does not
// depend on scheduling, so it is the same alone and in a batch.
//
// Each radix pass is three launches with no inter-block waiting:
//   hist     per-block digit histogram of a tile of 256, 1024 or 4096 keys -> hist[digit][block]
//   rowscan  one warp per digit: exclusive scan along the blocks, digit totals
//   scatter  per block: digit bases from the totals, then 1, 4 or 16 rounds of 256 keys,
//            ranking equal digits within a warp by __match_any_sync and across
//            warps by a per-digit prefix in shared memory (stable order:
//            round, warp, lane = particle order)
#include "sc_common.cuh"

namespace ocsc {

constexpr int RT = 256;
constexpr int RITEMS = 16;  // rounds of RT keys per block at most (large sorts)
constexpr int RWARPS = RT / 32;
constexpr int RMAXBITS = 9;
constexpr int RBINS = 1 << RMAXBITS;  // 512 digits at most
constexpr unsigned FULLM = 0xffffffffu;

__global__ void __launch_bounds__(RT) k_rhist(const uint32_t* __restrict__ keys, int64_t n, int shift, int bins,
                                              uint32_t* __restrict__ hist, int items) {
    pdl_wait();
    __shared__ uint32_t h[RBINS];
    for (int d = threadIdx.x; d < RBINS; d += RT) h[d] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RT * items;
    const uint32_t mask = (uint32_t)bins - 1;
#pragma unroll 4
    for (int it = 0; it < items; ++it) {
        const int64_t i = base + it * RT + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < bins; d += RT) hist[(size_t)d * gridDim.x + blockIdx.x] = h[d];
}

__global__ void k_rrowscan(uint32_t* __restrict__ hist, int nblk, int bins, uint32_t* __restrict__ tot) {
    pdl_wait();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= bins) return;
    uint32_t* row = hist + (size_t)warp * nblk;
    uint32_t carry = 0;
    for (int b0 = 0; b0 < nblk; b0 += 32) {
        const int b = b0 + lane;
        const uint32_t v = b < nblk ? row[b] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULLM, incl, o);
            if (lane >= o) incl += t;
        }
        if (b < nblk) row[b] = carry + incl - v;
        carry += __shfl_sync(FULLM, incl, 31);
    }
    if (lane == 0) tot[warp] = carry;
}

__global__ void __launch_bounds__(RT) k_rscatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                 int64_t n, int shift, int bins, const uint32_t* __restrict__ hist,
                                                 const uint32_t* __restrict__ tot, uint32_t* __restrict__ kout,
                                                 uint32_t* __restrict__ vout, const double* __restrict__ qsrc,
                                                 void* __restrict__ qout, int qfloat, int items) {
    pdl_wait();
    __shared__ uint32_t base[RBINS];
    __shared__ uint32_t wc[RWARPS][RBINS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // exclusive scan of the digit totals (at most 512, by warp 0) plus this
    // block's offset within each digit -> where the block's keys of a digit go
    if (warp == 0) {
        uint32_t carry = 0;
        for (int d0 = 0; d0 < bins; d0 += 32) {
            const int d = d0 + lane;
            const uint32_t v = d < bins ? tot[d] : 0u;
            uint32_t inc = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(FULLM, inc, o);
                if (lane >= o) inc += t;
            }
            if (d < bins) base[d] = carry + inc - v + hist[(size_t)d * gridDim.x + blockIdx.x];
            carry += __shfl_sync(FULLM, inc, 31);
        }
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t mask = (uint32_t)bins - 1;
    const int64_t tile = (int64_t)blockIdx.x * RT * items;
    for (int r = 0; r < items; ++r) {
        const int64_t i = tile + (int64_t)r * RT + tid;
        const bool valid = i < n;
        const uint32_t key = valid ? kin[i] : 0u;
        const uint32_t val = valid ? (vin ? vin[i] : (uint32_t)i) : 0u;
        const uint32_t d = valid ? ((key >> shift) & mask) : (uint32_t)RBINS;
        for (int dd = tid; dd < bins; dd += RT)
#pragma unroll
            for (int w = 0; w < RWARPS; ++w) wc[w][dd] = 0u;
        __syncthreads();
        const uint32_t peers = __match_any_sync(FULLM, d);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wc[warp][d] = __popc(peers);
        __syncthreads();
        for (int dd = tid; dd < bins; dd += RT) {
            uint32_t run = base[dd];
#pragma unroll
            for (int w = 0; w < RWARPS; ++w) {
                const uint32_t c = wc[w][dd];
                wc[w][dd] = run;
                run += c;
            }
            base[dd] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wc[warp][d] + rank;
            kout[pos] = key;
            if (qsrc) {  // last pass of the deposit: carry the charge itself
                const double qv = qsrc[val];
                if (qfloat) static_cast<float*>(qout)[pos] = (float)qv;
                else static_cast<double*>(qout)[pos] = qv;
            } else {
                vout[pos] = val;
            }
        }
        __syncthreads();
    }
}

// Rounds of RT keys per block: every round pays a clear and a scan of the
// digit table behind four barriers whatever its size, so small sorts take
// one or four rounds per block (more blocks in parallel) and large ones 16
// (fewer digit-table rows for the scans).  The stable order, and so the
// result, does not depend on the tiling.
static int sort_items(int64_t n) { return n <= (1 << 18) ? 1 : (n <= (1 << 20) ? 4 : RITEMS); }
int sort_blocks(int64_t n) {
    const int64_t t = (int64_t)RT * sort_items(n);
    return (int)((n + t - 1) / t);
}

int sort_passes(int key_bits) { return key_bits <= 0 ? 1 : (key_bits + RMAXBITS - 1) / RMAXBITS; }

size_t sort_scratch_bytes(int64_t n, int key_bits) {
    (void)key_bits;
    const size_t nb = (size_t)(sort_blocks(n) > 0 ? sort_blocks(n) : 1);
    return align_up(4 * (size_t)n) * 2 + align_up((size_t)RBINS * nb * 4) + align_up((size_t)RBINS * 4);
}

cudaError_t launch_sort(const uint32_t* keys_in, int64_t n, int key_bits, uint32_t* keys_out, uint32_t* perm_out,
                        uint32_t* tmp_k, uint32_t* tmp_v, uint32_t* hist, uint32_t* tot, cudaStream_t s,
                        const double* q_src, void* q_out, bool q_float) {
    if (n <= 0) return cudaSuccess;
    const int nb = sort_blocks(n), items = sort_items(n);
    const int passes = sort_passes(key_bits);
    const int width = key_bits <= 0 ? 1 : (key_bits + passes - 1) / passes;  // <= RMAXBITS
    const uint32_t* sk = keys_in;
    const uint32_t* sv = nullptr;
    bool to_out = (passes % 2) == 1;
    for (int p = 0; p < passes; ++p) {
        const int shift = width * p;
        int dbits = key_bits - shift;
        dbits = dbits > width ? width : (dbits < 1 ? 1 : dbits);
        const int bins = 1 << dbits;
        uint32_t* dk = to_out ? keys_out : tmp_k;
        uint32_t* dv = to_out ? perm_out : tmp_v;
        launch(k_rhist, nb, RT, 0, s, sk, n, shift, bins, hist, items);
        launch(k_rrowscan, (bins * 32 + 255) / 256, 256, 0, s, hist, nb, bins, tot);
        const bool last = p == passes - 1;
        launch(k_rscatter, nb, RT, 0, s, sk, sv, n, shift, bins, hist, tot, dk, dv, last ? q_src : nullptr,
                                     last ? q_out : nullptr, q_float ? 1 : 0, items);
        sk = dk;
        sv = dv;
        to_out = !to_out;
    }
    return cudaGetLastError();
}

// Cell bounds of the sorted runs: start[key] and end[key] (both 0 for an
// empty cell, from a memset).
__global__ void k_cell_bounds(const uint32_t* __restrict__ sk, int64_t n, uint32_t* __restrict__ start,
                              uint32_t* __restrict__ end, const ScState* st) {
    pdl_wait();
    if (st->status) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t key = sk[j];
        if (j == 0 || sk[j - 1] != key) start[key] = (uint32_t)j;
        if (j == n - 1 || sk[j + 1] != key) end[key] = (uint32_t)(j + 1);
    }
}

// The cell's run of charges, which the last radix pass carried into sorted
// (cell, particle) order, summed into the cell.  FP64: one thread per cell, a
// strictly sequential left fold in particle order from 0 -- np.bincount's
// summation (sc.py:193), bit for bit.  (One warp per cell with every lane
// folding the same shuffled values spent 32 lanes of this GPU's narrow FP64
// pipe per addition: 370 us per 2M particles.)  FP32: one warp per cell,
// lane-strided Kahan sums combined by a fixed shuffle tree with error-free
// (two-sum) additions.  Empty cells get 0, so no memset of the grid.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <typename R>
__global__ void __launch_bounds__(256) k_deposit_cells(const R* __restrict__ sq, const uint32_t* __restrict__ start,
                                                       const uint32_t* __restrict__ end, int64_t ncell,
                                                       R* __restrict__ qgrid, const ScState* st) {
    pdl_wait();
    if (st->status) return;
    if constexpr (sizeof(R) == 8) {
        const int64_t nt = (int64_t)gridDim.x * blockDim.x;
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell; c += nt) {
            const uint32_t b = start[c], e = end[c];
            double sum = 0.0;
            uint32_t k = b;
            for (; k + 4 <= e; k += 4) {  // four loads in flight, the additions in order
                const double v0 = sq[k], v1 = sq[k + 1], v2 = sq[k + 2], v3 = sq[k + 3];
                sum = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(sum, v0), v1), v2), v3);
            }
            for (; k < e; ++k) sum = __dadd_rn(sum, (double)sq[k]);
            qgrid[c] = (R)sum;
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = w0; c < ncell; c += nw) {
        const uint32_t b = start[c], e = end[c];
        {
            float sum = 0.f, comp = 0.f;
            for (uint32_t k = b + lane; k < e; k += 32) {
                const float y = __fsub_rn((float)sq[k], comp);
                const float t = __fadd_rn(sum, y);
                comp = __fsub_rn(__fsub_rn(t, sum), y);
                sum = t;
            }
            float err = -comp;
            for (int o = 16; o; o >>= 1) {
                const float s2 = __shfl_down_sync(0xffffffffu, sum, o);
                const float e2 = __shfl_down_sync(0xffffffffu, err, o);
                float ns, ne;
                two_sum(sum, s2, ns, ne);
                sum = ns;
                err = __fadd_rn(__fadd_rn(err, e2), ne);
            }
            if (lane == 0) qgrid[c] = (R)__fadd_rn(sum, err);
        }
    }
}

cudaError_t launch_deposit(const Plan& p, const Layout& L, char* ws, const double* q, int64_t n, cudaStream_t s) {
    (void)q;
    const ScState* st = reinterpret_cast<const ScState*>(ws + L.state);
    const int64_t ncell = (int64_t)p.nx * p.ny * p.nz;
    cudaError_t e = cudaMemsetAsync(ws + L.cell_start, 0, 2 * align_up(4 * (size_t)ncell), s);
    if (e) return e;
    int64_t b = (n + 255) / 256;
    if (b > (int64_t)p.sm_count * 8) b = (int64_t)p.sm_count * 8;
    if (b < 1) b = 1;
    const uint32_t* sk = reinterpret_cast<const uint32_t*>(ws + L.sort_keys);
    uint32_t* cs = reinterpret_cast<uint32_t*>(ws + L.cell_start);
    uint32_t* ce = reinterpret_cast<uint32_t*>(ws + L.cell_end);
    launch(k_cell_bounds, (int)b, 256, 0, s, sk, n, cs, ce, st);
    const int cb = p.prec == SC_FP64 ? (int)((ncell + 255) / 256 < (int64_t)p.sm_count * 16 ? (ncell + 255) / 256
                                                                                            : (int64_t)p.sm_count * 16)
                                     : p.sm_count * 8;
    if (p.prec == SC_FP64)
        launch(k_deposit_cells<double>, cb, 256, 0, s, reinterpret_cast<const double*>(ws + L.sort_q), cs, ce, ncell,
                                                   reinterpret_cast<double*>(ws + L.qgrid), st);
    else
        launch(k_deposit_cells<float>, cb, 256, 0, s, reinterpret_cast<const float*>(ws + L.sort_q), cs, ce, ncell,
                                                  reinterpret_cast<float*>(ws + L.qgrid), st);
    return cudaGetLastError();
}

}  // namespace ocsc
