// md_kernels.cu -- all device kernels of the engine and the C-ABI host code.
//
// Kernel map (reference function each one replaces, paths relative to the
// ls1-mardyn tree):
//   k_wrap              DomainDecompBase::handleDomainLeavingParticles (DomainDecompBase.cpp:199-249)
//   k_ref_cells         LinkedCells::getCellIndexOfPoint (LinkedCells.cpp:870-923)
//   k_halo_count        DomainDecompBase::populateHaloLayerWithCopies (DomainDecompBase.cpp:317-376):
//                       number of halo copies each molecule generates
//   k_list_hist/scan/   LinkedCells::update + FullParticleCell::buildSoACaches: counting sort
//   k_list_scatter/     of the molecules into cells, slots re-sorted into cell order
//   k_cell_sort/k_permute
//   k_build_list        C08CellPairTraversal over the 27-cell neighbourhood (C08CellPairTraversal.h,
//                       C08BasedTraversals.h:48-152) -> owner-computes pair-candidate list
//   k_sites             FullMolecule::setupSoACache (FullMolecule.cpp:711-767)
//   k_force_lj / k_force_ms
//                       VectorizedCellProcessor::_calculatePairs + _loopBody* (VCP.cpp:171-2730)
//                       fused with FullMolecule::calcFM (FullMolecule.cpp:548-631)
//   k_pre               FullMolecule::upd_preF (FullMolecule.cpp:331-361)
//   k_post              FullMolecule::upd_postF + Leapfrog::transition2to3 (Leapfrog.cpp:63-147)
//   k_finalize          VCP::endTraversal (VCP.cpp:122-155), Domain local sums
#include "md_device.cuh"
#include "md_pair.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <thread>

#include "../../include/ls1gb300.h"

using namespace md;

__constant__ Params cP;

// status word bits (device -> host)
#define ST_LOST 1u
#define ST_LIST_OVERFLOW 2u
#define ST_NAN 4u
#define ST_CELL_SORT 8u

struct Scratch {
    // reductions
    double* partials;       // [NPART][pstride], slot-major per-warp partials
    double* result;         // finalize output (NPART doubles)
    md_step_record* records;
    int* step;              // step counter for md_run records
    unsigned* status;
    unsigned* need_rebuild;
    unsigned* disp_max;     // float bits
    int* list_need;         // max candidates needed (overflow report)
};

#define NPART 32   // partial-sum slots per block
// slots: 0 upot6lj 1 upotXpoles 2 virial 3 myRF 4 mol_pairs 5..11 site pairs 12 summv2 13 sumIw2 14 n 15 rotdof
// 16..23 summv2 per component, 24..31 sumIw2 per component (component-wise thermostats only)
#define SLOT_MV2_C 16
#define SLOT_IW2_C 24

// ------------------------------------------------------------------ reductions
// Every kernel that contributes to the global sums writes, per warp of its
// grid, one partial per slot into a slot-major array partials[slot * pstride
// + warp]; all warps of the grid write (zeros where they own no molecule), so
// nothing needs clearing.  k_finalize sums each slot in a fixed order
// (deterministic) with one block per slot.
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void warp_partial(double* partials, int pstride, int slot, double v) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0)
        partials[(size_t)slot * pstride + ((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5)] = v;
}

// A slot this kernel contributes nothing to: lane 0 writes the zero partial
// without a reduction.
__device__ __forceinline__ void warp_partial_zero(double* partials, int pstride, int slot) {
    if ((threadIdx.x & 31) == 0)
        partials[(size_t)slot * pstride + ((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5)] = 0.0;
}

// FP64 instructions are scarce on this GPU: a warp-wide FP64 operation
// holds its sub-partition's FP64 pipe for about 64 cycles (measured: the
// FP64 pipe of a pair kernel was 53 % busy with 72 FP64 warp instructions
// per molecule).  The FP32 pair kernels therefore combine and convert their
// per-molecule and per-warp results with FP32 and integer instructions.

// Exact float -> double conversion on the integer pipes: sign, exponent
// re-biased by 1023 - 127, mantissa moved up by 52 - 23 bits.  Zero stays
// (signed) zero, subnormal floats (|x| < 1.18e-38) become zero, infinities
// and NaNs stay infinities and NaNs.
__device__ __forceinline__ double f2d_exact(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t ex = (b >> 23) & 0xffu;
    const uint64_t sign = (uint64_t)(b >> 31) << 63;
    const uint64_t man = (uint64_t)(b & 0x7fffffu) << 29;
    const uint64_t e64 = ex == 0xffu ? 0x7ffull : (uint64_t)(ex + 896u);
    const uint64_t r = ex == 0u ? sign : (sign | (e64 << 52) | man);
    return __longlong_as_double((long long)r);
}

// double -> float conversion, rounded to nearest even, on the integer pipes:
// the magnitude is rounded at the 29th bit (carries may reach the exponent),
// the exponent re-biased by 127 - 1023.  Results below FP32's normal range
// become (signed) zero, results above it infinity; NaN stays NaN.  Equal to
// the IEEE conversion for every input whose FP32 result is normal, zero,
// infinite or NaN.
__device__ __forceinline__ float d2f_int(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long mag = b & 0x7fffffffffffffffull;
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const unsigned long long m = mag + 0x0fffffffull + ((mag >> 29) & 1ull);
    const int e = (int)(m >> 52) - 896;
    uint32_t r = sign | ((uint32_t)e << 23) | ((uint32_t)(m >> 29) & 0x7fffffu);
    r = e >= 255 ? (sign | 0x7f800000u) : r;
    r = e <= 0 ? sign : r;
    r = mag > 0x7ff0000000000000ull ? 0x7fc00000u : r;
    return __uint_as_float(r);
}

// Error-free FP32 sum over the warp of per-lane values hi + lo: a butterfly
// whose every level adds the hi parts with TwoSum (Knuth) and carries the
// rounding error into lo.  Every lane ends with the same total hi + lo
// (TwoSum's error term is exact, so both partners of a level compute it
// alike), accurate to about 2^-44 relative.
__device__ __forceinline__ void twosum_xor(float& hi, float& lo, int o) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    const float s = __fadd_rn(hi, h2);
    const float bp = __fadd_rn(s, -hi);
    const float err = __fadd_rn(__fadd_rn(hi, -__fadd_rn(s, -bp)), __fadd_rn(h2, -bp));
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, l2), err);
}

__device__ __forceinline__ void warp_twosum(float& hi, float& lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) twosum_xor(hi, lo, o);
}

// Per-warp partial of an FP32 per-lane value: compensated FP32 warp sum,
// one FP64 addition (lane 0) to store hi + lo.
__device__ __forceinline__ void warp_partial_f32(double* partials, int pstride, int slot, float v) {
    float hi = v, lo = 0.f;
    warp_twosum(hi, lo);
    if ((threadIdx.x & 31) == 0)
        partials[(size_t)slot * pstride + ((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5)] =
            f2d_exact(hi) + f2d_exact(lo);
}

// Integer-valued partial (a pair count): reduced exactly in FP32 across the
// warp (|sum| < 2^24), converted once.
__device__ __forceinline__ void warp_partial_count(double* partials, int pstride, int slot, float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
        partials[(size_t)slot * pstride + ((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5)] = f2d_exact(v);
}

// Sum `v` over the block (blockDim multiple of 32, <= 1024); result valid in thread 0.
__device__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        int nw = blockDim.x >> 5;
        r = threadIdx.x < nw ? sh[threadIdx.x] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// slots 0..11 come from the force kernel (nw_force warps), 12..13 from the
// post-force half step (nw_post warps), 16..31 from the post-force half step
// when it writes per-component sums (nw_comp warps); a count of 0 leaves a
// slot at 0.  Stage 1: FIN_SEG blocks per slot each sum a contiguous
// segment; stage 2 sums the FIN_SEG segment sums of each slot in order
// (deterministic).
#define FIN_SEG 64
__global__ void k_finalize1(const double* partials, int pstride, int nw_force, int nw_post, int nw_rot, int nw_comp,
                            double* seg) {
    __shared__ double sh[32];
    const int s = blockIdx.y, b = blockIdx.x;
    const int nw = s < 12 ? nw_force : (s == 12 ? nw_post : (s == 13 ? nw_rot : (s >= SLOT_MV2_C ? nw_comp : 0)));
    if (nw == 0) {  // slot unused by this step (whole block leaves together)
        if (threadIdx.x == 0) seg[s * FIN_SEG + b] = 0.0;
        return;
    }
    const int per = (nw + FIN_SEG - 1) / FIN_SEG;
    const int lo = b * per, hi = min(nw, lo + per);
    double v = 0.0;
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) v += partials[(size_t)s * pstride + k];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) seg[s * FIN_SEG + b] = v;
}

// Second stage of the fixed-order sums (one warp, one slot per lane); with
// rec, also the step record (Upot, virial, sum m v^2, sum I w^2) of the
// step counted by *step.
__global__ void k_finalize2(const double* seg, double* result, md_step_record* rec, int* step, int has_rot_dof) {
    const int s = threadIdx.x;
    double v = 0.0;
    if (s < NPART)
        for (int b = 0; b < FIN_SEG; ++b) v += seg[s * FIN_SEG + b];
    if (s < NPART) result[s] = v;
    if (!rec) return;  // uniform over the warp
    const double u6 = __shfl_sync(0xffffffffu, v, 0), ux = __shfl_sync(0xffffffffu, v, 1);
    const double vir = __shfl_sync(0xffffffffu, v, 2), myRF = __shfl_sync(0xffffffffu, v, 3);
    const double mv2 = __shfl_sync(0xffffffffu, v, 12), iw2 = __shfl_sync(0xffffffffu, v, 13);
    if (s == 0) {
        const int k = *step;
        rec[k].upot = u6 / 6.0 + ux + myRF;
        rec[k].virial = vir + 3.0 * myRF;
        rec[k].summv2 = mv2;
        rec[k].sumIw2 = has_rot_dof ? iw2 : 0.0;
        *step = k + 1;
    }
}

// ------------------------------------------------------------------ wrap + cells
__device__ __forceinline__ double& coord(State& S, int d, int64_t i) {
    return d == 0 ? S.rx[i] : d == 1 ? S.ry[i] : S.rz[i];
}

// DomainDecompBase::handleDomainLeavingParticles for every periodic dimension:
// lower face first (shift +L, clamp below max), then upper face (shift -L,
// clamp to min).  Molecules further than rc outside the box are lost in the
// reference; they raise ST_LOST here.
__device__ void wrap_molecule(State& S, int64_t i, unsigned* status, unsigned long long* nwrapped) {
    double r[3] = {S.rx[i], S.ry[i], S.rz[i]};
    int moved = 0;
    for (int d = 0; d < 3; ++d) {
        if (!cP.periodic[d]) continue;
        double lo[3], hi[3];
        for (int e = 0; e < 3; ++e) { lo[e] = cP.bmin[e] - cP.rc; hi[e] = cP.bmax[e] + cP.rc; }
        // direction -: region [min - rc, min) in d
        bool inreg = true;
        for (int e = 0; e < 3; ++e) {
            double l = lo[e], h = (e == d) ? cP.bmin[d] : hi[e];
            inreg &= (r[e] >= l && r[e] < h);
        }
        if (inreg) {
            r[d] = r[d] + cP.L[d];
            if (r[d] >= cP.bmax[d]) r[d] = next_down(cP.bmax[d]);
            moved = 1;
        }
        inreg = true;
        for (int e = 0; e < 3; ++e) {
            double l = (e == d) ? cP.bmax[d] : lo[e], h = hi[e];
            inreg &= (r[e] >= l && r[e] < h);
        }
        if (inreg) {
            r[d] = r[d] + (-cP.L[d]);
            if (r[d] <= cP.bmin[d]) r[d] = cP.bmin[d];
            moved = 1;
        }
    }
    for (int d = 0; d < 3; ++d)
        if (cP.periodic[d] && !(r[d] >= cP.bmin[d] && r[d] < cP.bmax[d])) atomicOr(status, ST_LOST);
    if (moved) {
        S.rx[i] = r[0]; S.ry[i] = r[1]; S.rz[i] = r[2];
        atomicAdd(nwrapped, 1ull);
    }
}

__global__ void k_wrap(State S, unsigned* status, unsigned long long* nwrapped, const unsigned* need) {
    if (need && !*need) return;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    wrap_molecule(S, i, status, nwrapped);
}

// LinkedCells::getCellIndexOfPoint with the border table of
// CellBorderAndFlagManager::getBorder (arithmetic kept unfused).
__device__ int64_t ref_cell_of_point(const double* point, const double* border, int bstride) {
    int ci[3];
    double p[3] = {point[0], point[1], point[2]};
    for (int d = 0; d < 3; ++d) {
        if (p[d] <= cP.rhmin[d]) p[d] = __dadd_rn(p[d], __dmul_rn(cP.rcl[d], 0.5));
        else if (p[d] >= cP.rhmax[d]) p[d] = __dsub_rn(p[d], __dmul_rn(cP.rcl[d], 0.5));
        int c = (int)floor(__dmul_rn(__dsub_rn(p[d], cP.bmin[d]), cP.rclr[d])) + 1;
        c = max(0, min(c, cP.rcpd[d] - 1));
        ci[d] = c;
    }
    bool inside = true;
    for (int d = 0; d < 3; ++d)
        inside &= (border[d * bstride + ci[d]] <= p[d]) && (p[d] < border[d * bstride + ci[d] + 1]);
    if (!inside) {
        for (int d = 0; d < 3; ++d) {
            if (p[d] < border[d * bstride + ci[d]]) ci[d]--;
            else if (p[d] >= border[d * bstride + ci[d] + 1]) ci[d]++;
            // points outside the halo box (the reference asserts on these) stay in range
            ci[d] = max(0, min(ci[d], cP.rcpd[d] - 1));
        }
    }
    return ((int64_t)ci[2] * cP.rcpd[1] + ci[1]) * cP.rcpd[0] + ci[0];
}

__global__ void k_ref_cells(State S, const double* border, int bstride, int64_t* cell_out_upload_order,
                            unsigned* occupancy) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    double p[3] = {S.rx[i], S.ry[i], S.rz[i]};
    int64_t c = ref_cell_of_point(p, border, bstride);
    if (cell_out_upload_order) cell_out_upload_order[S.orig[i]] = c;
    if (occupancy) atomicAdd(&occupancy[c], 1u);
}

// Halo copies of DomainDecompBase::populateHaloLayerWithCopies: a molecule in
// [min, min+rc) or [max-rc, max) of a periodic dimension is copied there, and
// copies of earlier dimensions are copied again, so it generates
// prod_d (1 + near_d) - 1 copies; each copy is binned into its halo cell.
__global__ void k_halo(State S, const double* border, int bstride, unsigned long long* nhalo, unsigned* occupancy) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    double r[3] = {S.rx[i], S.ry[i], S.rz[i]};
    int sh[3];
    int cnt = 1;
    for (int d = 0; d < 3; ++d) {
        sh[d] = 0;
        if (!cP.periodic[d]) continue;
        if (r[d] >= cP.bmin[d] && r[d] < cP.bmin[d] + cP.rc) sh[d] = 1;
        else if (r[d] >= cP.bmax[d] - cP.rc && r[d] < cP.bmax[d]) sh[d] = -1;
        if (sh[d]) cnt *= 2;
    }
    if (cnt == 1) return;
    atomicAdd(nhalo, (unsigned long long)(cnt - 1));
    if (!occupancy) return;
    for (int m = 1; m < 8; ++m) {
        bool ok = true;
        double p[3];
        for (int d = 0; d < 3; ++d) {
            int use = (m >> d) & 1;
            if (use && !sh[d]) { ok = false; break; }
            p[d] = r[d];
            if (use) {
                if (sh[d] > 0) { p[d] = r[d] + cP.L[d]; if (p[d] < cP.bmax[d]) p[d] = next_up(cP.bmax[d]); }
                else { p[d] = r[d] + (-cP.L[d]); if (p[d] >= cP.bmin[d]) p[d] = next_down(cP.bmin[d]); }
            }
        }
        if (!ok) continue;
        atomicAdd(&occupancy[ref_cell_of_point(p, border, bstride)], 1u);
    }
}

__global__ void k_max_u32(const unsigned* a, int64_t n, unsigned* out) {
    unsigned m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, a[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ------------------------------------------------------------------ list-grid binning
__device__ __forceinline__ int list_cell_coord(double x, int d) {
    int c = (int)floor((x - cP.bmin[d]) * cP.linv[d]);
    return max(0, min(c, cP.ln[d] - 1));
}

__device__ void wrap_molecule(State& S, int64_t i, unsigned* status, unsigned long long* nwrapped);

// Leaving-particle wrap for molecules outside the box, then the list cell of
// every molecule and its histogram.
// With msub (the Newton-3 cluster path) also the octant of the list cell the
// molecule lies in, in Morton order (x bit 0, y bit 1, z bit 2), for the
// order inside the cell.
__global__ void k_list_hist(State S, int* mcell, int* counts, unsigned* status, unsigned long long* nwrapped,
                            const unsigned* need, unsigned char* msub) {
    if (!*need) return;
    // grid-stride (as the other rebuild kernels): a step that needs no rebuild launches few blocks to skip; not
    // unrolled, so that the registers stay those of one molecule per thread
#pragma unroll 1
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = S.rx[i], y = S.ry[i], z = S.rz[i];
    if (!(x >= cP.bmin[0] && x < cP.bmax[0] && y >= cP.bmin[1] && y < cP.bmax[1] && z >= cP.bmin[2] && z < cP.bmax[2]))
        wrap_molecule(S, i, status, nwrapped);
    int cx = list_cell_coord(S.rx[i], 0), cy = list_cell_coord(S.ry[i], 1), cz = list_cell_coord(S.rz[i], 2);
    int c = (cz * cP.ln[1] + cy) * cP.ln[0] + cx;
    mcell[i] = c;
    atomicAdd(&counts[c], 1);
    if (msub) {
        const int o[3] = {cx, cy, cz};
        const double r[3] = {S.rx[i], S.ry[i], S.rz[i]};
        unsigned char k = 0;
        for (int d = 0; d < 3; ++d)
            if ((r[d] - cP.bmin[d]) * cP.linv[d] - o[d] >= 0.5) k |= (unsigned char)(1u << d);
        msub[i] = k;
    }
    }
}

// Exclusive scan of counts[0..n) into start[0..n] (and cursor) in three
// passes: per-block sums, one block scanning the block sums, per-block scans.
#define SCAN_BLOCK 1024
__global__ void k_scan1(const int* counts, int n, int* bsum, const unsigned* need) {
    if (!*need) return;
    __shared__ int sh[32];
    int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    int v = i < n ? counts[i] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = sh[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) bsum[blockIdx.x] = v;
    }
}

__global__ void k_scan2(int* bsum, int nb, int* total_out, const unsigned* need) {
    if (!*need) return;
    __shared__ int sh[1024];
    int per = (nb + blockDim.x - 1) / blockDim.x;
    int b = threadIdx.x * per, e = min(nb, b + per);
    int s = 0;
    for (int k = b; k < e; ++k) s += bsum[k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        int v = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - s;
    for (int k = b; k < e; ++k) {
        int c = bsum[k];
        bsum[k] = run;
        run += c;
    }
    if (threadIdx.x == blockDim.x - 1) *total_out = sh[threadIdx.x];
}

__global__ void k_scan3(const int* counts, int n, const int* boff, int* start, int* cursor, const unsigned* need) {
    if (!*need) return;
    __shared__ int sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int i = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    int v = i < n ? counts[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = sh[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        sh[lane] = t;
    }
    __syncthreads();
    int excl = boff[blockIdx.x] + (w > 0 ? sh[w - 1] : 0) + x - v;
    if (i < n) {
        start[i] = excl;
        cursor[i] = excl;
    }
}

__global__ void k_list_scatter(int64_t n, const int* mcell, int* cursor, int* perm, const unsigned* need) {
    if (!*need) return;
#pragma unroll 1
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int p = atomicAdd(&cursor[mcell[i]], 1);
        perm[p] = (int)i;
    }
}

// Deterministic order inside each cell: one warp per cell ranks the cell's
// slot indices (the atomic scatter leaves them in arbitrary order) and writes
// them back sorted, by component first when `comp` is given (so the warps of
// the pair kernels see runs of one component), then by previous slot.  Cells
// of up to 64 molecules are ranked in registers; larger cells fall back to a
// serial insertion sort by lane 0.
// With msub (one component, the Newton-3 cluster path) by octant of the cell
// first, so that runs of consecutive slots are compact clusters.
__device__ __forceinline__ int cell_sort_key(const int* comp, const unsigned char* msub, int v) {
    return comp ? (comp[v] << MD_CODE_SHIFT) | v : (msub ? ((int)msub[v] << MD_CODE_SHIFT) | v : v);
}

__device__ __forceinline__ void cell_sort_one(const int* start, int* perm, const int* comp,
                                              const unsigned char* msub, int c, int lane);
__global__ void k_cell_sort(const int* start, int ncells, int* perm, const int* comp, const unsigned* need,
                            const unsigned char* msub) {
    if (!*need) return;
    const int lane = threadIdx.x & 31;
    const int nw = (int)((gridDim.x * (int64_t)blockDim.x) >> 5);
#pragma unroll 1
    for (int c = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5); c < ncells; c += nw) {
        cell_sort_one(start, perm, comp, msub, c, lane);
        __syncwarp();  // (lane 0 alone sorts cells of more than 64)
    }
}

// One cell of k_cell_sort (one warp): stable ranking by the sort key.
__device__ __forceinline__ void cell_sort_one(const int* start, int* perm, const int* comp,
                                              const unsigned char* msub, int c, int lane) {
    int b = start[c], e = start[c + 1], m = e - b;
    if (m <= 1) return;
    if (m <= 64) {
        int v0 = lane < m ? cell_sort_key(comp, msub, perm[b + lane]) : 0x7fffffff;
        int v1 = lane + 32 < m ? cell_sort_key(comp, msub, perm[b + lane + 32]) : 0x7fffffff;
        int r0 = 0, r1 = 0;
        for (int t = 0; t < 32; ++t) {
            int a0 = __shfl_sync(0xffffffffu, v0, t), a1 = __shfl_sync(0xffffffffu, v1, t);
            r0 += (a0 < v0) + (a1 < v0);
            r1 += (a0 < v1) + (a1 < v1);
        }
        __syncwarp();
        if (lane < m) perm[b + r0] = v0 & (int)MD_INDEX_MASK;
        if (lane + 32 < m) perm[b + r1] = v1 & (int)MD_INDEX_MASK;
        return;
    }
    if (lane == 0) {
        for (int k = b + 1; k < e; ++k) {
            const int v = perm[k], kv = cell_sort_key(comp, msub, v);
            int q = k - 1;
            while (q >= b && cell_sort_key(comp, msub, perm[q]) > kv) { perm[q + 1] = perm[q]; --q; }
            perm[q + 1] = v;
        }
    }
}

// Gather all master arrays into slot order (dst = src[perm]); the force
// outputs F, M, Vi only with `outputs`.
__global__ void k_permute(State dst, State src, const int* perm, const int* mcell, const unsigned* need, int outputs) {
    if (!*need) return;
    // one molecule per thread (a grid-stride loop here let the compiler overlap iterations at 80 registers,
    // and the gathers ran at a third of the occupancy)
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= src.n) return;
    int64_t i = perm[k];
#define PM(a) dst.a[k] = src.a[i]
    PM(rx); PM(ry); PM(rz); PM(vx); PM(vy); PM(vz); PM(qw); PM(qx); PM(qy); PM(qz); PM(Lx); PM(Ly); PM(Lz);
    if (outputs) {
        PM(Fx); PM(Fy); PM(Fz); PM(Mx); PM(My); PM(Mz); PM(Vx); PM(Vy); PM(Vz);
    }
    PM(comp); PM(orig); PM(id);
#undef PM
    dst.home[k] = mcell[i];
}

// Local coordinates relative to the home-cell origin.  At a list rebuild the
// origin (FP64) and the local coordinates then (FP32, for the displacement
// test) are stored per molecule; every pre-force step recomputes the local
// coordinates from the FP64 position.  Slot n gets a position far outside
// every box: candidate rows are padded with it.
__global__ void k_local(State S, float4* xlf, double* origin, float4* xlref, const unsigned* need,
                        float4* xl_other) {
    if (need && !*need) return;
#pragma unroll 1
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= S.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (i == S.n) {  // the far-away slot that pads candidate rows (in both local-coordinate buffers)
        xlf[i] = make_float4(1e18f, 1e18f, 1e18f, __int_as_float(0));
        if (xl_other) xl_other[i] = xlf[i];
        continue;
    }
    int h = S.home[i];
    int cx = h % cP.ln[0], cy = (h / cP.ln[0]) % cP.ln[1], cz = h / (cP.ln[0] * cP.ln[1]);
    double ox = cP.bmin[0] + cx * cP.lside[0], oy = cP.bmin[1] + cy * cP.lside[1], oz = cP.bmin[2] + cz * cP.lside[2];
    origin[3 * i] = ox; origin[3 * i + 1] = oy; origin[3 * i + 2] = oz;
    float4 p;
    p.x = d2f_int(S.rx[i] - ox);
    p.y = d2f_int(S.ry[i] - oy);
    p.z = d2f_int(S.rz[i] - oz);
    p.w = __int_as_float(S.comp[i]);
    xlf[i] = p;
    xlref[i] = p;
    }
}

// Pair-candidate rows of the thread-per-molecule kernels (single-centre LJ)
// in mixed precision are interleaved in 32-byte blocks (one DRAM sector) across the 32
// molecules of a warp: block c (entries 8c .. 8c + 7) of molecule i is block
// ((i / 32) * (maxnb / 8) + c) * 32 + i % 32 of the list, so the lanes of a
// warp read one kilobyte of consecutive bytes per block instead of one
// sector from each of 32 rows, and the list build writes whole sectors.
// The rows of the warp-per-molecule kernels (multi-site) and of the FP64
// kernels, which read one entry at a time, stay row-major (row i at
// i * maxnb).  maxnb is a multiple of 8.
__device__ __forceinline__ size_t il_block(int64_t i, int c, int maxnb) {
    return ((size_t)(i >> 5) * (size_t)(maxnb >> 3) + (size_t)c) * 32 + (size_t)(i & 31);
}
__device__ __forceinline__ size_t il_entry(int64_t i, int k, int maxnb) {
    return il_block(i, k >> 3, maxnb) * 8 + (size_t)(k & 7);
}
// 16-byte chunk q (entries 4q .. 4q + 3) of an interleaved row, relative to
// the row's first chunk
__device__ __forceinline__ int il_q(int q) { return (q >> 1) * 64 + (q & 1); }
// Entry k of a row relative to the row's entry 0 (interleaved or row-major).
template <bool IL>
__device__ __forceinline__ int row_off(int k) {
    return IL ? (k >> 3) * 256 + (k & 7) : k;
}

#define BL_WARPS 4
#define BL_BUF 8
// Geometry of one box's list grid: cells per axis, cell edges, periodicity,
// and the global index of its first cell (boxes of a batch are numbered one
// after another).
struct ListGrid {
    int ln[3];
    float side[3];
    bool per[3];
    int base;
};

// Tests this lane's molecule against the m staged candidates (negated,
// shifted coordinates sx/sy/sz, list entries se; slots m .. 31 far away when
// m < 32), two per paired FP32 instruction, and appends the hits to the
// lane's shared-memory buffer, flushing it to the row in 32-byte blocks.
template <bool IL>
__device__ __forceinline__ void test_staged(int m, const float2 pix, const float2 piy, const float2 piz, float rl2,
                                            const float* sx, const float* sy, const float* sz, const uint32_t* se,
                                            bool own, uint32_t self, uint32_t* buf, int& nb, int& cnt, uint32_t* row,
                                            int maxnb) {
    uint32_t hits = 0u;
    auto test2 = [&](int t) {
        const float2 dx = __fadd2_rn(pix, *reinterpret_cast<const float2*>(sx + t));
        const float2 dy = __fadd2_rn(piy, *reinterpret_cast<const float2*>(sy + t));
        const float2 dz = __fadd2_rn(piz, *reinterpret_cast<const float2*>(sz + t));
        float2 r2 = __fmul2_rn(dz, dz);
        r2 = __ffma2_rn(dy, dy, r2);
        r2 = __ffma2_rn(dx, dx, r2);
        hits |= (r2.x < rl2 ? 1u : 0u) << t;
        hits |= (r2.y < rl2 ? 1u : 0u) << (t + 1);
    };
    if (m == 32) {  // a full staging area (the common case): bit positions known at compile time
#pragma unroll
        for (int t = 0; t < 32; t += 2) test2(t);
    } else {
        const int mm = (m + 1) & ~1;  // pairs of staged slots; slot m (if odd) is far away
#pragma unroll 4
        for (int t = 0; t < mm; t += 2) test2(t);
    }
    if (!own) hits = 0u;
    while (hits) {
        const int t = __ffs(hits) - 1;
        hits &= hits - 1u;
        const uint32_t en = se[t];
        if (en == self) continue;  // not the molecule itself
        buf[nb++] = en;
        if (nb == BL_BUF) {
            if (cnt + BL_BUF <= maxnb) {
                uint4* dst = reinterpret_cast<uint4*>(row + row_off<IL>(cnt));
                dst[0] = make_uint4(buf[0], buf[1], buf[2], buf[3]);
                dst[1] = make_uint4(buf[4], buf[5], buf[6], buf[7]);
            } else {
                for (int u = 0; u < BL_BUF && cnt + u < maxnb; ++u) row[row_off<IL>(cnt + u)] = buf[u];
            }
            cnt += BL_BUF;
            nb = 0;
        }
    }
}

// Rows of the molecules of list cell `lc` (local index in grid g), built by
// one warp; sq (4 x 32 words) and sbuf are this warp's shared-memory areas.
// For up to 32 home molecules at a time (one per lane) the warp streams the
// candidates of the 27 neighbour cells in order; a candidate farther from
// the bounding box of the home molecules than the list radius (enlarged by
// a relative 1e-4, so FP32 rounding cannot drop a pair the exact test
// keeps) is skipped, the others are compacted into a staging area of 32
// (negated coordinates shifted into the home cell's frame, and their list
// entries), and every full staging area is tested by all lanes at once.
// The rows keep the candidates in neighbour-cell and slot order.
template <bool IL>
__device__ __forceinline__ void build_cell_rows(int64_t n, const float4* xl, const int* start, const ListGrid& g,
                                                int lc, uint32_t* nbr, int* nnb, int maxnb, float rl2,
                                                unsigned* status, int* need_max, float* sq,
                                                uint32_t (*sbuf)[BL_BUF + 1], int lane) {
    const int hc[3] = {lc % g.ln[0], (lc / g.ln[0]) % g.ln[1], lc / (g.ln[0] * g.ln[1])};
    const int c = g.base + lc;
    const int b = start[c], e = start[c + 1];
    uint32_t* buf = sbuf[lane];
    float* sx = sq;
    float* sy = sq + 32;
    float* sz = sq + 64;
    uint32_t* se = reinterpret_cast<uint32_t*>(sq + 96);
    const float pre2 = rl2 * 1.0001f;
    for (int i0 = b; i0 < e; i0 += 32) {
        const int i = i0 + lane;
        const bool own = i < e;
        float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
        if (own) pi = xl[i];
        const float2 pix = make_float2(pi.x, pi.x), piy = make_float2(pi.y, pi.y), piz = make_float2(pi.z, pi.z);
        // bounding box of this group of home molecules
        float lox = own ? pi.x : 3.0e38f, loy = own ? pi.y : 3.0e38f, loz = own ? pi.z : 3.0e38f;
        float hix = own ? pi.x : -3.0e38f, hiy = own ? pi.y : -3.0e38f, hiz = own ? pi.z : -3.0e38f;
        for (int o = 16; o > 0; o >>= 1) {
            lox = fminf(lox, __shfl_xor_sync(0xffffffffu, lox, o));
            loy = fminf(loy, __shfl_xor_sync(0xffffffffu, loy, o));
            loz = fminf(loz, __shfl_xor_sync(0xffffffffu, loz, o));
            hix = fmaxf(hix, __shfl_xor_sync(0xffffffffu, hix, o));
            hiy = fmaxf(hiy, __shfl_xor_sync(0xffffffffu, hiy, o));
            hiz = fmaxf(hiz, __shfl_xor_sync(0xffffffffu, hiz, o));
        }
        const uint32_t self = (uint32_t)i | (13u << MD_CODE_SHIFT);
        int cnt = 0, nb = 0, fill = 0;
        const int64_t il = own ? i : 0;
        uint32_t* row = IL ? nbr + il_block(il, 0, maxnb) * 8 : nbr + (size_t)il * maxnb;
        for (int oz = -1; oz <= 1; ++oz)
            for (int oy = -1; oy <= 1; ++oy)
                for (int ox = -1; ox <= 1; ++ox) {
                    const int o[3] = {ox, oy, oz};
                    int cc[3];
                    bool skip = false;
                    for (int d = 0; d < 3; ++d) {
                        cc[d] = hc[d] + o[d];
                        if (cc[d] < 0 || cc[d] >= g.ln[d]) {
                            if (!g.per[d]) { skip = true; break; }
                            cc[d] = (cc[d] + g.ln[d]) % g.ln[d];
                        }
                    }
                    if (skip) continue;
                    const int cell = g.base + (cc[2] * g.ln[1] + cc[1]) * g.ln[0] + cc[0];
                    const uint32_t code = (uint32_t)((ox + 1) + 3 * (oy + 1) + 9 * (oz + 1));
                    const float shx = ox * g.side[0], shy = oy * g.side[1], shz = oz * g.side[2];
                    const int nb0 = start[cell], ne = start[cell + 1];
                    for (int j0 = nb0; j0 < ne; j0 += 32) {
                        const int jj = j0 + lane;
                        bool keep = false;
                        float x = 0.f, y = 0.f, z = 0.f;
                        if (jj < ne) {
                            const float4 pj = xl[jj];
                            x = pj.x + shx;
                            y = pj.y + shy;
                            z = pj.z + shz;
                            const float dx = fmaxf(fmaxf(lox - x, x - hix), 0.f);
                            const float dy = fmaxf(fmaxf(loy - y, y - hiy), 0.f);
                            const float dz = fmaxf(fmaxf(loz - z, z - hiz), 0.f);
                            keep = dx * dx + dy * dy + dz * dz < pre2;
                        }
                        const uint32_t mk = __ballot_sync(0xffffffffu, keep);
                        const int ck = __popc(mk), rank = __popc(mk & ((1u << lane) - 1u));
                        const int room = 32 - fill;
                        const uint32_t en = (uint32_t)jj | (code << MD_CODE_SHIFT);
                        if (keep && rank < room) {
                            sx[fill + rank] = -x;
                            sy[fill + rank] = -y;
                            sz[fill + rank] = -z;
                            se[fill + rank] = en;
                        }
                        if (ck >= room) {  // the staging area is full: test it, then stage the rest
                            __syncwarp();
                            test_staged<IL>(32, pix, piy, piz, rl2, sx, sy, sz, se, own, self, buf, nb, cnt, row,
                                            maxnb);
                            __syncwarp();
                            if (keep && rank >= room) {
                                sx[rank - room] = -x;
                                sy[rank - room] = -y;
                                sz[rank - room] = -z;
                                se[rank - room] = en;
                            }
                            fill = ck - room;
                        } else {
                            fill += ck;
                        }
                    }
                }
        // the last, partial staging area (unused slots far away)
        __syncwarp();
        if (lane >= fill) {
            sx[lane] = 1e18f;
            sy[lane] = 1e18f;
            sz[lane] = 1e18f;
        }
        __syncwarp();
        if (fill > 0)
            test_staged<IL>(fill, pix, piy, piz, rl2, sx, sy, sz, se, own, self, buf, nb, cnt, row, maxnb);
        __syncwarp();  // the next group reuses the staging area
        if (own) {
            for (int u = 0; u < nb && cnt + u < maxnb; ++u) row[row_off<IL>(cnt + u)] = buf[u];
            cnt += nb;
            // pad the row to a multiple of four with the far-away slot n (zero cell offset)
            const uint32_t pad = (uint32_t)n | (13u << MD_CODE_SHIFT);
            for (int u = cnt; u < ((cnt + 3) & ~3) && u < maxnb; ++u) row[row_off<IL>(u)] = pad;
            nnb[i] = min(cnt, maxnb);
            if (cnt > maxnb) {
                atomicOr(status, ST_LIST_OVERFLOW);
                atomicMax(need_max, cnt);
            }
        }
    }
}

// Owner-computes pair-candidate list over the 27 list cells around each
// molecule's home cell (periodic wrap in periodic dimensions).  One warp per
// home cell holds up to 32 of its molecules, one per lane.  For each
// neighbour cell the warp stages 32 candidates at a time in shared memory
// (coalesced load, already shifted into the home cell's frame); every lane
// tests its molecule against the staged candidates (broadcast reads, two
// per paired FP32 instruction) and appends hits to its own 8-entry
// shared-memory buffer, flushed as one 32-byte block into its row (IL:
// interleaved rows for the thread-per-molecule kernels, else row-major).
// Candidate test in FP32 local coordinates against
// (rc + skin)^2 enlarged by a relative 2e-4, so no pair that can come within
// rc before the next rebuild is missed.
template <bool IL>
__global__ void __launch_bounds__(BL_WARPS * 32, 8) k_build_list(int64_t n, const float4* xl, const int* start,
                                                              int ncells, uint32_t* nbr, int* nnb, int maxnb,
                                                              float rl2, unsigned* status, int* need_max,
                                                              const unsigned* need) {
    if (!*need) return;
    __shared__ __align__(16) float sq[BL_WARPS][4][32];
    __shared__ uint32_t sbuf[BL_WARPS][32][BL_BUF + 1];  // +1: no bank conflicts between lanes
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    ListGrid g;
    for (int d = 0; d < 3; ++d) {
        g.ln[d] = cP.ln[d];
        g.side[d] = (float)cP.lside[d];
        g.per[d] = cP.periodic[d] != 0;
    }
    g.base = 0;
    // warp-stride over the cells (warp-uniform; only warp-level synchronisation below)
#pragma unroll 1
    for (int c = blockIdx.x * BL_WARPS + wl; c < ncells; c += gridDim.x * BL_WARPS)
        build_cell_rows<IL>(n, xl, start, g, c, nbr, nnb, maxnb, rl2, status, need_max, &sq[wl][0][0], sbuf[wl],
                            lane);
}

// ------------------------------------------------------------------ site cache
// FullMolecule::setupSoACache: normalise q, rotate site offsets and
// orientations.  Offsets are stored relative to the molecule centre.
template <typename Real>
__global__ void k_sites(State S, Real* sd, Real* se, int stride) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const CompDev& C = cP.comp[S.comp[i]];
    double w = S.qw[i], x = S.qx[i], y = S.qy[i], z = S.qz[i];
    // (CUDA's FP64 rsqrt: within an ulp of 1 / sqrt, one call where sqrt and a division each take several FP64
    // instructions on GB300's slow FP64 pipe; the reference divides by the norm, which rounds differently anyway)
    double s = rsqrt(w * w + x * x + y * y + z * z);
    w *= s; x *= s; y *= s; z *= s;
    S.qw[i] = w; S.qx[i] = x; S.qy[i] = y; S.qz[i] = z;
    if constexpr (sizeof(Real) == 4) {
        // FP32 caches: the rotation in FP32 from the normalised FP64 quaternion (rounded on the integer pipes;
        // GB300's FP64 rate made the FP64 rotations most of this kernel's time)
        const float wf = d2f_int(w), xf = d2f_int(x), yf = d2f_int(y), zf = d2f_int(z);
        for (int k = 0; k < C.ns; ++k) {
            float o[3];
            qrotf(wf, xf, yf, zf, C.df[k], o);
            for (int e = 0; e < 3; ++e) sd[((int64_t)i * stride + k) * MD_SITE_VEC + e] = (Real)o[e];
            if (C.kind[k] >= SK_DIPOLE) {
                qrotf(wf, xf, yf, zf, C.ef[k], o);
                for (int e = 0; e < 3; ++e) se[((int64_t)i * stride + k) * MD_SITE_VEC + e] = (Real)o[e];
            }
        }
    } else {
        for (int k = 0; k < C.ns; ++k) {
            double o[3];
            qrot(w, x, y, z, C.d[k], o);
            for (int e = 0; e < 3; ++e) sd[((int64_t)i * stride + k) * MD_SITE_VEC + e] = (Real)o[e];
            if (C.kind[k] >= SK_DIPOLE) {
                qrot(w, x, y, z, C.e[k], o);
                for (int e = 0; e < 3; ++e) se[((int64_t)i * stride + k) * MD_SITE_VEC + e] = (Real)o[e];
            }
        }
    }
}

// ------------------------------------------------------------------ forces
// FP64 image shift of neighbour j seen from i for cell-offset code `code`:
// the reference's halo copy r_j +- L.
__device__ __forceinline__ void image_shift(int h, uint32_t code, double* sh) {
    int hc[3] = {h % cP.ln[0], (h / cP.ln[0]) % cP.ln[1], h / (cP.ln[0] * cP.ln[1])};
    for (int d = 0; d < 3; ++d) {
        int c = hc[d] + decode_o(code, d);
        sh[d] = c < 0 ? -cP.L[d] : (c >= cP.ln[d] ? cP.L[d] : 0.0);
    }
}

__device__ __forceinline__ double fp64_r2(const State& S, int64_t i, int64_t j, uint32_t code) {
    double sh[3];
    image_shift(S.home[i], code, sh);
    double dx = S.rx[i] - (S.rx[j] + sh[0]);
    double dy = S.ry[i] - (S.ry[j] + sh[1]);
    double dz = S.rz[i] - (S.rz[j] + sh[2]);
    return __dadd_rn(__dmul_rn(dx, dx), __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dz, dz)));
}

// Single-LJ-centre molecules (centre at the molecule origin), FP32 pair
// arithmetic: the hot kernel of the 1CLJ benchmarks.  One thread per
// molecule streams its candidate row four entries per 16-byte load, gathers
// the four neighbour positions before computing (latency hiding), re-decides
// pairs within 4e-6 relative of a cut-off in FP64, and accumulates F with
// Kahan compensation; Vi, Upot and virial are plain FP32 per molecule and
// FP64 across molecules.
__global__ void __launch_bounds__(256, 4) k_force_lj32(State S, const float4* __restrict__ xlf,
                                                       const uint32_t* __restrict__ nbr, const int* __restrict__ nnb,
                                                       int maxnb, double* partials, int pstride) {
    __shared__ float4 soff[27];
    if (threadIdx.x < 27) {
        int t = threadIdx.x;
        soff[t] = make_float4((float)((t % 3 - 1) * cP.lside[0]), (float)(((t / 3) % 3 - 1) * cP.lside[1]),
                              (float)((t / 9 - 1) * cP.lside[2]), 0.f);
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    KSum fx, fy, fz;
    fx.init(); fy.init(); fz.init();
    float vx = 0.f, vy = 0.f, vz = 0.f, up = 0.f, vir = 0.f;
    int npairs = 0, nmol = 0;
    if (i < S.n) {
        const float4 p4 = xlf[i];
        const int ci = __float_as_int(p4.w);
        const int gi = cP.comp[ci].ljoff;
        const int cnt = nnb[i];
        const float rclj2 = cP.rclj2f, rc2 = cP.rc2f;
        const float band_lj = cP.band_hi_lj - cP.rclj2f, band_rc = cP.band_hi - cP.rc2f;
        const bool one_comp = cP.ncomp == 1, same_cut = cP.rc2 == cP.rclj2;
        float e24 = cP.eps24f[gi * cP.nlj + gi], s2 = cP.sig2f[gi * cP.nlj + gi];
        float sh6 = cP.shift6f[gi * cP.nlj + gi];
        int cur = gi;
        const uint4* row = reinterpret_cast<const uint4*>(nbr + il_block(i, 0, maxnb) * 8);
        for (int k = 0; k < cnt; k += 4) {
            const uint4 e4 = __ldg(row + il_q(k >> 2));
            const uint32_t ee[4] = {e4.x, e4.y, e4.z, e4.w};
            float4 pj[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) pj[t] = __ldg(&xlf[(k + t < cnt) ? (ee[t] & MD_INDEX_MASK) : i]);
            float gx = 0.f, gy = 0.f, gz = 0.f;  // this group's force, added compensated below
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (k + t >= cnt) break;
                const int j = (int)(ee[t] & MD_INDEX_MASK);
                const float4 o = soff[ee[t] >> MD_CODE_SHIFT];
                const float dx = (p4.x - pj[t].x) - o.x;
                const float dy = (p4.y - pj[t].y) - o.y;
                const float dz = (p4.z - pj[t].z) - o.z;
                const float r2 = dx * dx + (dy * dy + dz * dz);
                const bool macro = j > i;
                bool in = r2 < rclj2;
                if (same_cut) {
                    if (fabsf(r2 - rclj2) < band_lj) in = fp64_r2(S, i, j, ee[t] >> MD_CODE_SHIFT) < cP.rclj2;
                } else {
                    bool in_rc = r2 < rc2;
                    if (fabsf(r2 - rclj2) < band_lj || fabsf(r2 - rc2) < band_rc) {
                        const double r2d = fp64_r2(S, i, j, ee[t] >> MD_CODE_SHIFT);
                        in = r2d < cP.rclj2;
                        in_rc = r2d < cP.rc2;
                    }
                    nmol += (in_rc && macro) ? 1 : 0;
                }
                if (!in) continue;
                if (!one_comp) {
                    const int gj = cP.comp[__float_as_int(pj[t].w)].ljoff;
                    if (gj != cur) {
                        cur = gj;
                        e24 = cP.eps24f[gi * cP.nlj + gj];
                        s2 = cP.sig2f[gi * cP.nlj + gj];
                        sh6 = cP.shift6f[gi * cP.nlj + gj];
                    }
                }
                // VCP::_loopBodyLJ: scale = eps24 / r^2 (2 lj12 - lj6)
                const float r2inv = __fdividef(1.0f, r2);
                const float lj2 = s2 * r2inv;
                const float lj6 = lj2 * lj2 * lj2;
                const float lj12m6 = lj6 * lj6 - lj6;
                const float scale = e24 * r2inv * (lj6 * lj6 + lj12m6);
                const float f0 = dx * scale, f1 = dy * scale, f2 = dz * scale;
                gx += f0; gy += f1; gz += f2;
                const float V0 = dx * f0, V1 = dy * f1, V2 = dz * f2;
                vx += V0; vy += V1; vz += V2;
                if (macro) {
                    up += e24 * lj12m6 + sh6;
                    vir += V0 + V1 + V2;
                    ++npairs;
                }
            }
            fx.add(gx); fy.add(gy); fz.add(gz);
        }
        if (same_cut) nmol = npairs;
        S.Fx[i] = f2d_exact(fx.s - fx.c); S.Fy[i] = f2d_exact(fy.s - fy.c); S.Fz[i] = f2d_exact(fz.s - fz.c);
        S.Mx[i] = 0.0; S.My[i] = 0.0; S.Mz[i] = 0.0;
        S.Vx[i] = f2d_exact(0.5f * vx); S.Vy[i] = f2d_exact(0.5f * vy); S.Vz[i] = f2d_exact(0.5f * vz);
    }
    warp_partial_f32(partials, pstride, 0, up);
    warp_partial_zero(partials, pstride, 1);
    warp_partial_f32(partials, pstride, 2, vir);
    warp_partial_zero(partials, pstride, 3);
    warp_partial_count(partials, pstride, 4, (float)nmol);
    warp_partial_count(partials, pstride, 5, (float)npairs);
    for (int sl = 6; sl < 12; ++sl) warp_partial_zero(partials, pstride, sl);
}

// FP64 re-decision of a pair near a cut-off, always evaluated in the frame of
// the pair's smaller slot index, so that the two directions of a pair decide
// alike (code 26 - c is the opposite cell offset of code c).
__device__ __forceinline__ double fp64_r2_canon(const State& S, int i, int j, uint32_t code) {
    return j > i ? fp64_r2(S, i, j, code) : fp64_r2(S, j, i, 26u - code);
}

// Candidate-row loads of the LJ kernels: rows are read sequentially, 16 bytes
// at a time, with an L2 prefetch-size hint of 256 bytes; the kernels load the
// next chunk one iteration ahead.
__device__ __forceinline__ uint4 ld_row_chunk(const uint4* p) {
    uint4 r;
    asm("ld.global.nc.L2::256B.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// One candidate pair of the packed LJ loop below: lanes .x and .y of every
// float2 are two different neighbours of the same molecule.  All arithmetic
// between the distance and the accumulators runs on Blackwell's paired FP32
// instructions (FFMA2/FADD2/FMUL2: two FP32 results per issue).  Pairs
// outside the cut-off are masked (scale 0), not branched around.
struct LjPack {
    float2 gx, gy, gz;        // this group's force / eps24
    float2 vx, vy, vz;        // sum d o f / eps24 over the molecule's pairs
    float2 up, nin;           // sum (lj12 - lj6), in-cut-off pair count
};

// Candidates whose FP32 r^2 lies within the FP64 re-decision band of the
// cut-off are left out of the packed loop and handled after it (keeping the
// FP64 code out of the loop's register budget): up to MD_AMB of them are
// remembered; with more, the row is scanned again for them.
#define MD_AMB 4
struct AmbList {
    uint32_t e[MD_AMB];
    int n;
};

__device__ __forceinline__ void amb_push(AmbList& am, uint32_t e) {
    if (am.n < MD_AMB) am.e[am.n] = e;
    ++am.n;
}

// The LJ pair of a deferred candidate found inside the cut-off, in the
// packed loop's formulas (eps24 factored out), added to lane .x.
__device__ __forceinline__ void lj_one(float dx, float dy, float dz, float r2, float s2, KSum& fx, KSum& fy, KSum& fz,
                                       LjPack& a) {
    const float r2i = rcp_approx(r2);
    const float nlj2 = -s2 * r2i;
    const float nlj6 = (nlj2 * nlj2) * nlj2;
    const float u = fmaf(nlj6, nlj6, nlj6);
    const float w = fmaf(nlj6, nlj6, u);
    const float sc = r2i * w;
    const float f0 = dx * sc, f1 = dy * sc, f2 = dz * sc;
    fx.add(f0); fy.add(f1); fz.add(f2);
    a.vx.x = fmaf(dx, f0, a.vx.x);
    a.vy.x = fmaf(dy, f1, a.vy.x);
    a.vz.x = fmaf(dz, f2, a.vz.x);
    a.up.x += u;
    a.nin.x += 1.f;
}

// FP32 squared distance with the packed loop's operation order:
// d = (p_i - p_j) + o per axis, r^2 = dx dx + (dy dy + dz dz) fused.
__device__ __forceinline__ float r2_scalar(const float4 pi, const float4 pj, float ox, float oy, float oz, float& dx,
                                           float& dy, float& dz) {
    dx = __fadd_rn(fmaf(pj.x, -1.f, pi.x), ox);
    dy = __fadd_rn(fmaf(pj.y, -1.f, pi.y), oy);
    dz = __fadd_rn(fmaf(pj.z, -1.f, pi.z), oz);
    float r2 = __fmul_rn(dz, dz);
    r2 = fmaf(dy, dy, r2);
    return fmaf(dx, dx, r2);
}

__device__ __forceinline__ void lj_pack2(const float2 pix, const float2 piy, const float2 piz,
                                         const float4 pa, const float4 pb, const float2 ox, const float2 oy,
                                         const float2 oz, uint32_t ea, uint32_t eb, const float2 ns2, const float rc2f,
                                         const float band, LjPack& a, AmbList& am) {
    const float2 m1 = make_float2(-1.f, -1.f);
    float2 dx = __ffma2_rn(make_float2(pa.x, pb.x), m1, pix);
    float2 dy = __ffma2_rn(make_float2(pa.y, pb.y), m1, piy);
    float2 dz = __ffma2_rn(make_float2(pa.z, pb.z), m1, piz);
    dx = __fadd2_rn(dx, ox);
    dy = __fadd2_rn(dy, oy);
    dz = __fadd2_rn(dz, oz);
    float2 r2 = __fmul2_rn(dz, dz);
    r2 = __ffma2_rn(dy, dy, r2);
    r2 = __ffma2_rn(dx, dx, r2);
    bool ina = r2.x < rc2f, inb = r2.y < rc2f;
    const bool nera = fabsf(r2.x - rc2f) < band, nerb = fabsf(r2.y - rc2f) < band;
    if (nera || nerb) {  // decided in FP64 after the loop
        if (nera) { ina = false; amb_push(am, ea); }
        if (nerb) { inb = false; amb_push(am, eb); }
    }
    const float2 msk = make_float2(ina ? 1.f : 0.f, inb ? 1.f : 0.f);
    const float2 r2i = make_float2(rcp_approx(r2.x), rcp_approx(r2.y));
    // VCP::_loopBodyLJ with eps24 factored out: u = lj12 - lj6, scale = (2 lj12 - lj6) / r^2
    const float2 nlj2 = __fmul2_rn(ns2, r2i);            // -sigma^2 / r^2
    const float2 nlj6 = __fmul2_rn(__fmul2_rn(nlj2, nlj2), nlj2);  // -lj6
    const float2 u = __ffma2_rn(nlj6, nlj6, nlj6);
    const float2 w = __ffma2_rn(nlj6, nlj6, u);
    const float2 sc = __fmul2_rn(__fmul2_rn(r2i, msk), w);
    const float2 f0 = __fmul2_rn(dx, sc), f1 = __fmul2_rn(dy, sc), f2 = __fmul2_rn(dz, sc);
    a.gx = __fadd2_rn(a.gx, f0);
    a.gy = __fadd2_rn(a.gy, f1);
    a.gz = __fadd2_rn(a.gz, f2);
    a.vx = __ffma2_rn(dx, f0, a.vx);
    a.vy = __ffma2_rn(dy, f1, a.vy);
    a.vz = __ffma2_rn(dz, f2, a.vz);
    a.up = __ffma2_rn(u, msk, a.up);
    a.nin = __fadd2_rn(a.nin, msk);
}

// Time-step constants of the half steps, computed on the host: dt/2 and
// dt/(2m) per component, the latter with the same IEEE division the
// reference performs per molecule (a device FP64 division costs about ten
// FP64 instructions per molecule, and FP64 throughput bounds these kernels).
struct Kick {
    double dt, dt_halve;
    double dtInv2m[MD_MAXC];
    float massf[MD_MAXC];
};

// dt/(2m) of component c by selects over the parameter (a dynamic index
// into a kernel parameter would copy it to local memory)
__device__ __forceinline__ double kick_dtInv2m(const Kick& K, int c) {
    double r = K.dtInv2m[0];
#pragma unroll
    for (int k = 1; k < MD_MAXC; ++k) r = c == k ? K.dtInv2m[k] : r;
    return r;
}
__device__ __forceinline__ float kick_massf(const Kick& K, int c) {
    float r = K.massf[0];
#pragma unroll
    for (int k = 1; k < MD_MAXC; ++k) r = c == k ? K.massf[k] : r;
    return r;
}

// Single-component, single-LJ-centre molecules with rc_lj = rc (the 1CLJ
// benchmarks), FP32 pair arithmetic on paired FP32 instructions.  One thread
// per molecule streams its candidate row 16 bytes (four entries) at a time;
// rows are padded to a multiple of four with an entry that points at a far
// away position (slot n), so the loop has no bounds tests.  Every pair is
// evaluated from both sides with identical rounding (the FP32 distance is
// antisymmetric and near-cut-off pairs are re-decided in one canonical
// frame), so Upot, virial and the pair count are half the per-molecule
// sums over all neighbours.  Force sums are Kahan-compensated per group of
// four candidates; eps24 multiplies the sums once per molecule.
//
// Epilogues: EPI_STORE writes F, M (zero) and Vi into the state.  EPI_RMM is
// the reduced memory mode's cell processor (VCP1CLJRMM.cpp:240-369): no force
// is stored, the kick v += dt_inv_m F is applied at once (dt_inv_m = dt / m,
// halved for the initial force pass), and with sum_v2 the kernel also
// contributes sum v.v of the kicked velocities (VelocityCellProcessorRMM.h:
// 95-128, no mass) to slot 12.  EPI_LEAPFROG is Leapfrog's post-force half
// step of this step fused with the pre-force half step of the next (the
// operations of k_post_pre in the same order; no force is stored): v and
// sum m v^2 (slot 12) as k_post, then the kick, the drift r' = r + dt v into
// the other position buffer (the near-cut-off FP64 decisions of other
// molecules read this step's positions in the same launch) and the local
// coordinates of r' into the other local-coordinate buffer, with the
// displacement since the last list build.
#define EPI_STORE 0
#define EPI_RMM 1
#define EPI_LEAPFROG 2
// EPI_RMM_DRIFT: EPI_RMM followed by the next step's drift r' = r + dt v
// (PositionCellProcessorRMM) into the other position buffer, as EPI_LEAPFROG
// writes its drift (dt = E.K.dt).
#define EPI_RMM_DRIFT 3
struct LfStep {
    Kick K;
    double *rx, *ry, *rz;  // positions of the next step (written)
    float4* xl;            // local coordinates of the next step (written)
    const double* origin;
    const float4* xlref;
    unsigned* disp_max;
};
// v.v of the reduced mode's velocity sums (one expression for every kernel
// that forms it, so their per-warp partials agree bit for bit)
__device__ __forceinline__ double rmm_v2(double x, double y, double z) { return x * x + y * y + z * z; }
#ifndef MD_LJX2_MIN_BLOCKS
#define MD_LJX2_MIN_BLOCKS 3  // blocks of 256 per SM the register budget is sized for
#endif
template <int EPI>
__global__ void __launch_bounds__(256, MD_LJX2_MIN_BLOCKS) k_force_lj32x2(State S, const float4* __restrict__ xlf,
                                                         const uint32_t* __restrict__ nbr,
                                                         const int* __restrict__ nnb, int maxnb, double* partials,
                                                         int pstride, double dt_inv_m, int sum_v2, LfStep E) {
    __shared__ float smax[8];
    // minus the offset of the neighbour cell's origin (code) from the home cell's origin, one table per
    // axis: three conflict-free 4-byte shared loads per candidate move fewer shared-memory wavefronts
    // than one 16-byte load (which also conflicts between codes 8 apart)
    __shared__ float nsx[32], nsy[32], nsz[32];
    if (threadIdx.x < 32) {
        const int t = threadIdx.x < 27 ? threadIdx.x : 13;
        nsx[threadIdx.x] = (float)(-(t % 3 - 1) * cP.lside[0]);
        nsy[threadIdx.x] = (float)(-((t / 3) % 3 - 1) * cP.lside[1]);
        nsz[threadIdx.x] = (float)(-(t / 9 - 1) * cP.lside[2]);
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float up = 0.f, vir = 0.f, npairs = 0.f;  // halved per-molecule sums (every pair is seen twice)
    float v2f = 0.f;                          // EPI_RMM: v.v after the kick; EPI_LEAPFROG: m v.v
    float d2 = 0.f;                           // EPI_LEAPFROG: squared displacement since the list build
    if (i < S.n) {
        const float4 p4 = xlf[i];
        const int gi = cP.comp[__float_as_int(p4.w)].ljoff;
        const float e24 = cP.eps24f[gi * cP.nlj + gi], s2 = cP.sig2f[gi * cP.nlj + gi];
        const float sh6 = cP.shift6f[gi * cP.nlj + gi];
        const float2 pix = make_float2(p4.x, p4.x), piy = make_float2(p4.y, p4.y), piz = make_float2(p4.z, p4.z);
        const float2 ns2 = make_float2(-s2, -s2);
        const float rc2f = cP.rclj2f, band = cP.band_hi_lj - cP.rclj2f;
        const int cnt = nnb[i];
        KSum fx, fy, fz;
        fx.init(); fy.init(); fz.init();
        LjPack a;
        a.vx = a.vy = a.vz = a.up = a.nin = make_float2(0.f, 0.f);
        AmbList am;
        am.n = 0;
        const uint4* row = reinterpret_cast<const uint4*>(nbr + il_block(i, 0, maxnb) * 8);
        uint4 nx = cnt > 0 ? ld_row_chunk(row) : make_uint4(0u, 0u, 0u, 0u);
        for (int k = 0; k < cnt; k += 4) {
            const uint4 e4 = nx;
            if (k + 4 < cnt) nx = ld_row_chunk(row + il_q((k >> 2) + 1));
            const float4 pa = __ldg(&xlf[e4.x & MD_INDEX_MASK]), pb = __ldg(&xlf[e4.y & MD_INDEX_MASK]);
            const float4 pc = __ldg(&xlf[e4.z & MD_INDEX_MASK]), pd = __ldg(&xlf[e4.w & MD_INDEX_MASK]);
            a.gx = a.gy = a.gz = make_float2(0.f, 0.f);
            const uint32_t ca = e4.x >> MD_CODE_SHIFT, cb = e4.y >> MD_CODE_SHIFT;
            const uint32_t cc = e4.z >> MD_CODE_SHIFT, cd = e4.w >> MD_CODE_SHIFT;
            lj_pack2(pix, piy, piz, pa, pb, make_float2(nsx[ca], nsx[cb]), make_float2(nsy[ca], nsy[cb]),
                     make_float2(nsz[ca], nsz[cb]), e4.x, e4.y, ns2, rc2f, band, a, am);
            lj_pack2(pix, piy, piz, pc, pd, make_float2(nsx[cc], nsx[cd]), make_float2(nsy[cc], nsy[cd]),
                     make_float2(nsz[cc], nsz[cd]), e4.z, e4.w, ns2, rc2f, band, a, am);
            fx.add(a.gx.x + a.gx.y);
            fy.add(a.gy.x + a.gy.y);
            fz.add(a.gz.x + a.gz.y);
        }
        if (am.n > 0) {  // near-cut-off candidates: FP64 decision in the canonical frame
            const bool listed = am.n <= MD_AMB;
            const int m = listed ? am.n : cnt;
            for (int t = 0; t < m; ++t) {
                const uint32_t en = listed ? am.e[t] : nbr[il_entry(i, t, maxnb)];
                const int j = (int)(en & MD_INDEX_MASK);
                const uint32_t code = en >> MD_CODE_SHIFT;
                float dx, dy, dz;
                const float r2 = r2_scalar(p4, __ldg(&xlf[j]), nsx[code], nsy[code], nsz[code], dx, dy, dz);
                if (!(fabsf(r2 - rc2f) < band)) continue;  // (row scan) not near the cut-off
                if (fp64_r2_canon(S, i, j, code) < cP.rclj2) lj_one(dx, dy, dz, r2, s2, fx, fy, fz, a);
            }
        }
        // epilogue in FP32 (the precision of the pair sums) with exact conversions to the FP64 state; the
        // products are rounded on their own (no contraction into the sums below), so every epilogue variant
        // forms the virial alike
        const float nin = a.nin.x + a.nin.y;
        const float vx = __fmul_rn(e24, a.vx.x + a.vx.y), vy = __fmul_rn(e24, a.vy.x + a.vy.y),
                    vz = __fmul_rn(e24, a.vz.x + a.vz.y);
        if (EPI == EPI_STORE) {
            S.Fx[i] = f2d_exact(e24 * (fx.s - fx.c));
            S.Fy[i] = f2d_exact(e24 * (fy.s - fy.c));
            S.Fz[i] = f2d_exact(e24 * (fz.s - fz.c));
            S.Mx[i] = 0.0; S.My[i] = 0.0; S.Mz[i] = 0.0;
            S.Vx[i] = f2d_exact(0.5f * vx); S.Vy[i] = f2d_exact(0.5f * vy); S.Vz[i] = f2d_exact(0.5f * vz);
        } else if (EPI == EPI_RMM || EPI == EPI_RMM_DRIFT) {
            const double ux = S.vx[i] + dt_inv_m * f2d_exact(e24 * (fx.s - fx.c));
            const double uy = S.vy[i] + dt_inv_m * f2d_exact(e24 * (fy.s - fy.c));
            const double uz = S.vz[i] + dt_inv_m * f2d_exact(e24 * (fz.s - fz.c));
            S.vx[i] = ux; S.vy[i] = uy; S.vz[i] = uz;
            const float gx = d2f_int(ux), gy = d2f_int(uy), gz = d2f_int(uz);
            v2f = gx * gx + (gy * gy + gz * gz);
            if (EPI == EPI_RMM_DRIFT) {
                const double dt = E.K.dt;
                const double rx = S.rx[i] + dt * ux, ry = S.ry[i] + dt * uy, rz = S.rz[i] + dt * uz;
                E.rx[i] = rx; E.ry[i] = ry; E.rz[i] = rz;
                const float4 q0 = E.xlref[i];
                float4 p;
                p.x = d2f_int(rx - E.origin[3 * i]);
                p.y = d2f_int(ry - E.origin[3 * i + 1]);
                p.z = d2f_int(rz - E.origin[3 * i + 2]);
                p.w = q0.w;
                E.xl[i] = p;
                const float ddx = p.x - q0.x, ddy = p.y - q0.y, ddz = p.z - q0.z;
                d2 = ddx * ddx + ddy * ddy + ddz * ddz;
            }
        } else {
            const double F[3] = {f2d_exact(e24 * (fx.s - fx.c)), f2d_exact(e24 * (fy.s - fy.c)),
                                 f2d_exact(e24 * (fz.s - fz.c))};
            const double h = E.K.dtInv2m[0], dt = E.K.dt;  // one component
            double v[3] = {S.vx[i], S.vy[i], S.vz[i]};
            for (int d = 0; d < 3; ++d) v[d] += h * F[d];
            const float gx = d2f_int(v[0]), gy = d2f_int(v[1]), gz = d2f_int(v[2]);
            v2f = E.K.massf[0] * (gx * gx + (gy * gy + gz * gz));
            for (int d = 0; d < 3; ++d) v[d] = v[d] + h * F[d];
            const double rx = S.rx[i] + dt * v[0], ry = S.ry[i] + dt * v[1], rz = S.rz[i] + dt * v[2];
            S.vx[i] = v[0]; S.vy[i] = v[1]; S.vz[i] = v[2];
            E.rx[i] = rx; E.ry[i] = ry; E.rz[i] = rz;
            const float4 q0 = E.xlref[i];
            float4 p;
            p.x = d2f_int(rx - E.origin[3 * i]);
            p.y = d2f_int(ry - E.origin[3 * i + 1]);
            p.z = d2f_int(rz - E.origin[3 * i + 2]);
            p.w = q0.w;
            E.xl[i] = p;
            const float ddx = p.x - q0.x, ddy = p.y - q0.y, ddz = p.z - q0.z;
            d2 = ddx * ddx + ddy * ddy + ddz * ddz;
        }
        up = 0.5f * (__fmul_rn(e24, a.up.x + a.up.y) + __fmul_rn(sh6, nin));
        vir = 0.5f * (vx + (vy + vz));
        npairs = 0.5f * nin;
    }
    warp_partial_f32(partials, pstride, 0, up);
    warp_partial_zero(partials, pstride, 1);
    warp_partial_f32(partials, pstride, 2, vir);
    warp_partial_zero(partials, pstride, 3);
    warp_partial_count(partials, pstride, 4, npairs);
    warp_partial_count(partials, pstride, 5, npairs);
    for (int sl = 6; sl < 12; ++sl) warp_partial_zero(partials, pstride, sl);
    if ((EPI == EPI_RMM || EPI == EPI_RMM_DRIFT) && sum_v2) warp_partial_f32(partials, pstride, 12, v2f);
    if (EPI == EPI_LEAPFROG || EPI == EPI_RMM_DRIFT) {
        if (EPI == EPI_LEAPFROG) warp_partial_f32(partials, pstride, 12, v2f);
        for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, o));
        if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = d2;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, smax[w]);
            atomicMax(E.disp_max, __float_as_uint(m));
        }
    }
}

// FP64 variant: absolute FP64 positions with the reference's halo image
// shift r_j +- L, FP64 arithmetic and accumulation throughout; epilogues as
// in k_force_lj32x2.
template <int EPI>
__global__ void __launch_bounds__(256) k_force_lj64(State S, const float4* __restrict__ xlf,
                                                    const uint32_t* __restrict__ nbr, const int* __restrict__ nnb,
                                                    int maxnb, double* partials, int pstride, double dt_inv_m,
                                                    int sum_v2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fx = 0, fy = 0, fz = 0, vx = 0, vy = 0, vz = 0, up = 0, vir = 0;
    double v2 = 0.0;  // EPI_RMM: v.v after the kick
    int npairs = 0, nmol = 0;
    if (i < S.n) {
        const int ci = S.comp[i];
        const int gi = cP.comp[ci].ljoff;
        const double pix = S.rx[i], piy = S.ry[i], piz = S.rz[i];
        const int h = S.home[i];
        const int cnt = nnb[i];
        for (int k = 0; k < cnt; ++k) {
            const uint32_t e = __ldg(nbr + (size_t)i * maxnb + k);  // FP64 mode: row-major rows
            const int j = (int)(e & MD_INDEX_MASK);
            const uint32_t code = e >> MD_CODE_SHIFT;
            double shf[3];
            image_shift(h, code, shf);
            const double dx = pix - (S.rx[j] + shf[0]);
            const double dy = piy - (S.ry[j] + shf[1]);
            const double dz = piz - (S.rz[j] + shf[2]);
            const double r2 = dx * dx + (dy * dy + dz * dz);
            const bool macro = j > i;
            nmol += (r2 < cP.rc2 && macro) ? 1 : 0;
            if (!(r2 < cP.rclj2)) continue;
            const int gj = cP.comp[S.comp[j]].ljoff;
            double f[3], V[3], u;
            const double d[3] = {dx, dy, dz};
            lj_pair<double>(d, d, r2, cP.eps24[gi * cP.nlj + gj], cP.sig2[gi * cP.nlj + gj], cP.shift6[gi * cP.nlj + gj],
                            f, V, u);
            fx += f[0]; fy += f[1]; fz += f[2];
            vx += V[0]; vy += V[1]; vz += V[2];
            if (macro) {
                up += u;
                vir += V[0] + V[1] + V[2];
                ++npairs;
            }
        }
        if (EPI == EPI_STORE) {
            S.Fx[i] = fx; S.Fy[i] = fy; S.Fz[i] = fz;
            S.Mx[i] = 0.0; S.My[i] = 0.0; S.Mz[i] = 0.0;
            S.Vx[i] = 0.5 * vx; S.Vy[i] = 0.5 * vy; S.Vz[i] = 0.5 * vz;
        } else {
            const double ux = S.vx[i] + dt_inv_m * fx, uy = S.vy[i] + dt_inv_m * fy, uz = S.vz[i] + dt_inv_m * fz;
            S.vx[i] = ux; S.vy[i] = uy; S.vz[i] = uz;
            v2 = rmm_v2(ux, uy, uz);
        }
    }
    warp_partial(partials, pstride, 0, up);
    warp_partial_zero(partials, pstride, 1);
    warp_partial(partials, pstride, 2, vir);
    warp_partial_zero(partials, pstride, 3);
    warp_partial_count(partials, pstride, 4, (float)nmol);
    warp_partial_count(partials, pstride, 5, (float)npairs);
    for (int sl = 6; sl < 12; ++sl) warp_partial_zero(partials, pstride, sl);
    if (EPI == EPI_RMM && sum_v2) warp_partial(partials, pstride, 12, v2);
}

// ---------------------------------------------------------------- multi-site
// Multi-site molecules are processed one warp per molecule: the warp's lanes
// share the molecule's component (its site loops are warp-uniform), and the
// candidate rows are stably partitioned by the neighbour's component after
// every list build, so consecutive candidates also share the neighbour's site
// loops.  The candidates inside a cut-off are compacted into a per-warp ring
// in row order before the site-pair work, so no lane idles on a candidate
// beyond the cut-off.

// Stable partition of every candidate row by the neighbour's component (one
// warp per molecule; the row is staged in dynamic shared memory, maxnb
// entries per warp).  Only the order within a row changes.
#define ROW_PART_SMEM (48 * 1024)  // shared bytes per block of k_row_partition (rows staged whole)
#define ROW_PART_BYTES(maxnb) ((int64_t)(maxnb) * 5)  // per row: the entries and a one-byte part key each

// With nhalf (the multi-site kernels' Newton-3 form) each row is first split
// into the neighbours in higher slots and those in lower slots, each part
// partitioned by component; nhalf[i] = the length of the first part.
__device__ __forceinline__ void row_partition_one(const float4* __restrict__ xl, uint32_t* nbr, const int* nnb,
                                                  int maxnb, int ncomp, int* nhalf, uint32_t* rowbuf, int wl,
                                                  int lane, int64_t i);
__global__ void k_row_partition(int64_t n, const float4* __restrict__ xl, uint32_t* nbr, const int* nnb, int maxnb,
                                int ncomp, const unsigned* need, int* nhalf) {
    if (!*need) return;
    extern __shared__ uint32_t rowbuf[];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll 1
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + wl; i < n; i += (int64_t)gridDim.x * (blockDim.x >> 5))
        row_partition_one(xl, nbr, nnb, maxnb, ncomp, nhalf, rowbuf, wl, lane, i);
}

// One row of k_row_partition (one warp; its staging areas at rowbuf).
__device__ __forceinline__ void row_partition_one(const float4* __restrict__ xl, uint32_t* nbr, const int* nnb,
                                                  int maxnb, int ncomp, int* nhalf, uint32_t* rowbuf, int wl,
                                                  int lane, int64_t i) {
    uint32_t* buf = rowbuf + (size_t)wl * maxnb;
    // each entry's part (lower half x ncomp + the neighbour's component), found once
    uint8_t* key = reinterpret_cast<uint8_t*>(rowbuf + (size_t)(blockDim.x >> 5) * maxnb) + (size_t)wl * maxnb;
    uint32_t* row = nbr + (size_t)i * maxnb;
    const int cnt = nnb[i];
    for (int k = lane; k < cnt; k += 32) {
        const uint32_t e = row[k];
        const int64_t j = e & MD_INDEX_MASK;
        const int c = ncomp == 1 ? 0 : __float_as_int(__ldg(&xl[j]).w);
        buf[k] = e;
        key[k] = (uint8_t)((nhalf && j < i ? ncomp : 0) + c);
    }
    __syncwarp();
    int out = 0;
    const int parts = nhalf ? 2 : 1;
    for (int h = 0; h < parts; ++h) {
        for (int c = 0; c < ncomp; ++c) {
            const int want = h * ncomp + c;
            for (int k0 = 0; k0 < cnt; k0 += 32) {
                const int k = k0 + lane;
                const bool m = k < cnt && key[k] == want;
                const unsigned bal = __ballot_sync(0xffffffffu, m);
                if (m) row[out + __popc(bal & ((1u << lane) - 1u))] = buf[k];
                out += __popc(bal);
            }
        }
        if (nhalf && h == 0 && lane == 0) nhalf[i] = out;
    }
}

// x, y, z of one site record of the site caches (one 16-byte load in FP32,
// a 16-byte and an 8-byte load in FP64; records are MD_SITE_VEC-aligned).
template <typename Real> __device__ __forceinline__ void site_rec(const Real* p, Real* o);
template <> __device__ __forceinline__ void site_rec<float>(const float* p, float* o) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z;
}
template <> __device__ __forceinline__ void site_rec<double>(const double* p, double* o) {
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    o[0] = v.x; o[1] = v.y; o[2] = __ldg(p + 2);
}

// Centre distance m_d = r_i - (r_j + image) of candidate e: FP32 local
// coordinates with the cell offset (mixed precision) or FP64 positions with
// the reference's halo shift.
template <typename Real>
__device__ __forceinline__ void ms_centre_distance(const State& S, const float4* xlf, const Real (*soff)[3],
                                                   const Real* pi, int64_t i, uint32_t e, Real* md) {
    const int64_t j = e & MD_INDEX_MASK;
    const uint32_t code = e >> MD_CODE_SHIFT;
    if (sizeof(Real) == 4) {
        const float4 pj = __ldg(&xlf[j]);
        md[0] = (pi[0] - (Real)pj.x) - soff[code][0];
        md[1] = (pi[1] - (Real)pj.y) - soff[code][1];
        md[2] = (pi[2] - (Real)pj.z) - soff[code][2];
    } else {
        double shf[3];
        image_shift(S.home[i], code, shf);
        md[0] = pi[0] - (S.rx[j] + shf[0]);
        md[1] = pi[1] - (S.ry[j] + shf[1]);
        md[2] = pi[2] - (S.rz[j] + shf[2]);
    }
}

// Cut-off flags of a candidate (bit 0: inside rc_lj, bit 1: inside rc); in
// mixed precision FP32 r^2 near a cut-off is re-decided in FP64 in the
// pair's canonical frame.
template <typename Real>
__device__ __forceinline__ int ms_flags(const State& S, int64_t i, uint32_t e, const Real* md) {
    const Real r2 = md[0] * md[0] + (md[1] * md[1] + md[2] * md[2]);
    const Real rclj2 = sizeof(Real) == 4 ? (Real)cP.rclj2f : (Real)cP.rclj2;
    const Real rc2 = sizeof(Real) == 4 ? (Real)cP.rc2f : (Real)cP.rc2;
    bool lj_on = r2 < rclj2, el_on = r2 < rc2;
    if (sizeof(Real) == 4) {
        const bool bl = r2 > (Real)cP.band_lo_lj && r2 < (Real)cP.band_hi_lj;
        const bool be = r2 > (Real)cP.band_lo && r2 < (Real)cP.band_hi;
        if (bl || be) {
            const double r2d = fp64_r2_canon(S, i, e & MD_INDEX_MASK, e >> MD_CODE_SHIFT);
            if (bl) lj_on = r2d < cP.rclj2;
            if (be) el_on = r2d < cP.rc2;
        }
    }
    return (lj_on ? 1 : 0) | (el_on ? 2 : 0);
}

// Walk molecule i's candidate row with the whole warp: each lane tests one
// candidate per round; candidates inside a cut-off enter the warp's ring of
// 64 (entry + flags) in row order; every full group of 32 is handed to
// `body(entry, flags, m_d)`, one candidate per lane, and the rest (< 32) at
// the end to the lanes below the count.
template <typename Real, typename Body>
__device__ __forceinline__ void ms_walk_row(const State& S, const float4* xlf, const Real (*soff)[3], const Real* pi,
                                            int64_t i, const uint32_t* row, int cnt, uint32_t* ring, int lane,
                                            Body body) {
    int head = 0, qn = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int k0 = 0; k0 < cnt; k0 += 32) {
        const int k = k0 + lane;
        int fl = 0;
        uint32_t e = 0u;
        if (k < cnt) {
            e = __ldg(&row[k]);
            Real md[3];
            ms_centre_distance<Real>(S, xlf, soff, pi, i, e, md);
            fl = ms_flags<Real>(S, i, e, md);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, fl != 0);
        if (fl) {
            const int p = (head + qn + __popc(bal & lt)) & 63;
            ring[p] = e;
            ring[64 + p] = (uint32_t)fl;
        }
        qn += __popc(bal);
        __syncwarp();
        if (qn >= 32) {
            const int p = (head + lane) & 63;
            const uint32_t ee = ring[p];
            const int ff = (int)ring[64 + p];
            __syncwarp();
            head = (head + 32) & 63;
            qn -= 32;
            Real md[3];
            ms_centre_distance<Real>(S, xlf, soff, pi, i, ee, md);
            body(ee, ff, md);
        }
    }
    if (qn > 0) {
        const int p = (head + lane) & 63;
        const uint32_t ee = ring[p];
        const int ff = (int)ring[64 + p];
        __syncwarp();
        if (lane < qn) {
            Real md[3];
            ms_centre_distance<Real>(S, xlf, soff, pi, i, ee, md);
            body(ee, ff, md);
        }
    }
    __syncwarp();
}

// Total over the warp of a per-lane compensated FP32 sum (rounded to FP32,
// the precision of the pair arithmetic) or plain FP64 sum; valid in lane 0.
// `scale` is a power of two (exact).
__device__ __forceinline__ double warp_total(const KSum& k, float scale = 1.f) {
    float hi = scale * k.s, lo = -scale * k.c;
    warp_twosum(hi, lo);
    return f2d_exact(__fadd_rn(hi, lo));
}
__device__ __forceinline__ double warp_total(const DSum& k, float scale = 1.f) { return (double)scale * warp_sum(k.s); }
// The same for a plain per-lane value.
__device__ __forceinline__ double warp_total_plain(float x, float scale = 1.f) {
    float hi = scale * x, lo = 0.f;
    warp_twosum(hi, lo);
    return f2d_exact(__fadd_rn(hi, lo));
}
__device__ __forceinline__ double warp_total_plain(double x, float scale = 1.f) { return (double)scale * warp_sum(x); }

// Per-warp partial of a per-lane accumulator, times sign (+-1).
__device__ __forceinline__ void warp_partial_acc(double* partials, int pstride, int slot, const KSum& k, float sign) {
    float hi = sign * k.s, lo = -sign * k.c;
    warp_twosum(hi, lo);
    if ((threadIdx.x & 31) == 0)
        partials[(size_t)slot * pstride + ((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5)] =
            f2d_exact(hi) + f2d_exact(lo);
}
__device__ __forceinline__ void warp_partial_acc(double* partials, int pstride, int slot, const DSum& k, float sign) {
    warp_partial(partials, pstride, slot, (double)sign * k.s);
}

#define MS_WARPS 4     // warps per block of the multi-site kernels
static_assert(MD_SITE_VEC * MD_MAXS <= 32, "one lane per element loads the warp molecule's site records");
#define MS_MOLS 32     // molecules per warp, one after another
#ifndef MS_MIN_BLOCKS
#define MS_MIN_BLOCKS 6  // FP32 force kernel: blocks per SM the register budget is sized for (80 registers, no spills)
#endif
#ifndef MS_ADJ_MIN_BLOCKS
#define MS_ADJ_MIN_BLOCKS 5  // FP32 adjoint kernel: the same (96 registers, no spills)
#endif
#ifndef MS_ADJ_N3_MIN_BLOCKS
// FP32 Newton-3 adjoint kernel: 72 registers, spills of 8-128 bytes per instance; measured on the
// 100,000-molecule mixture 0.559 ms against 0.579 ms at 6 blocks (80 registers) and 0.633 ms at 5 (96)
#define MS_ADJ_N3_MIN_BLOCKS 7
#endif
#define MS_ADJ_MIN_MOLS 8  // fewest molecules per warp of the multi-site adjoint
#ifndef MS_N3_MIN_BLOCKS
#define MS_N3_MIN_BLOCKS 5  // FP32 Newton-3 force kernel, general signatures: the same (96 registers, no spills)
#endif
#ifndef MS2_N3_MIN_BLOCKS
// FP32 Newton-3 two-component kernel: 72 registers, a 16-byte spill; measured at the 1M mixture 1.59 ms
// against 1.63 ms at 6 blocks (80 registers), 1.75 ms at 5 (92) and more spills at 8
#define MS2_N3_MIN_BLOCKS 7
#endif

// Site signature of a component as the multi-site kernels read it (sites in
// the order LJ centres, charges, dipoles, quadrupoles): SigDyn reads the
// component's table at run time; SigFix<ID, NL, NC, ND, NQ, LJOFF, LJTOT>
// states component ID's counts, the global index of its first LJ centre and
// the system's number of LJ centres at compile time, so that the site-pair
// loops of a molecule pair unroll into straight code with no kind dispatch
// and constant parameter-table offsets.
struct SigDyn {
    const CompDev& c;
    int id;
    __device__ __forceinline__ int nlj() const { return c.nlj; }
    __device__ __forceinline__ int nch() const { return c.nch; }
    __device__ __forceinline__ int ndi() const { return c.ndi; }
    __device__ __forceinline__ int nqu() const { return c.nqu; }
    __device__ __forceinline__ int ns() const { return c.ns; }
    __device__ __forceinline__ int ljoff() const { return c.ljoff; }
    __device__ __forceinline__ int ljtot() const { return cP.nlj; }
    __device__ __forceinline__ int kind(int a) const { return c.kind[a]; }
    __device__ __forceinline__ int comp() const { return id; }
};
template <int ID, int NL, int NC, int ND, int NQ, int LJOFF, int LJTOT>
struct SigFix {
    __device__ __forceinline__ static constexpr int nlj() { return NL; }
    __device__ __forceinline__ static constexpr int nch() { return NC; }
    __device__ __forceinline__ static constexpr int ndi() { return ND; }
    __device__ __forceinline__ static constexpr int nqu() { return NQ; }
    __device__ __forceinline__ static constexpr int ns() { return NL + NC + ND + NQ; }
    __device__ __forceinline__ static constexpr int ljoff() { return LJOFF; }
    __device__ __forceinline__ static constexpr int ljtot() { return LJTOT; }
    __device__ __forceinline__ static constexpr int kind(int a) {
        return a < NL ? SK_LJ : a < NL + NC ? SK_CHARGE : a < NL + NC + ND ? SK_DIPOLE : SK_QUAD;
    }
    __device__ __forceinline__ static constexpr int comp() { return ID; }
};

// Signature dispatch by component index: DispDyn hands `f` the run-time
// signature; DispFix2<S0, S1> the compile-time one of a two-component system;
// DispOne<S0> always S0 (kernels launched for one component's molecules).
struct DispDyn {
    template <class F>
    __device__ __forceinline__ static void run(int c, F f) { f(SigDyn{cP.comp[c], c}); }
};
template <class S0>
struct DispOne {
    template <class F>
    __device__ __forceinline__ static void run(int, F f) { f(S0()); }
};
template <class S0, class S1>
struct DispFix2 {
    template <class F>
    __device__ __forceinline__ static void run(int c, F f) {
        if (c == 0) f(S0());
        else f(S1());
    }
};

// Pair counts by kind of one warp (molecule pairs, LJ, C-C, C-D, D-D, C-Q, D-Q, Q-Q).
struct MsCounts {
    int mol = 0, lj = 0, cc = 0, cd = 0, dd = 0, cq = 0, dq = 0, qq = 0;
};

// One molecule pair: the LJ x LJ site pairs, then each electrostatic site of
// the home molecule (A) against the charges, dipoles and quadrupoles of the
// neighbour (B), one body per kind pair.  The home-site forces are summed per
// site before its lever-arm torque; the virial of the molecule pair is
// m_d o (sum of its site forces).  fp, mp: force and torque on the home
// molecule; u6p, uxp, rfp: its LJ (times 6), multipole and reaction-field
// energies.  With N3 also mq, the torque on the neighbour about its centre
// (the reference's Newton-3 half of processCellPair, VCP.cpp:2744-2819):
// per site pair f_a x d_b (the force -f_a acts at the neighbour's site
// offset d_b) plus the body's multipole torque on site b.
template <typename Real, bool N3 = false, class SA, class SB>
__device__ __forceinline__ void ms_molpair(const SA& A, const SB& B, const Real (*da_t)[3], const Real (*ea_t)[3],
                                           const Real* sd, const Real* se, uint32_t jb, const Real* md, int fl,
                                           bool macro, Real epsRF, Real* fp, Real* mp, Real* mq, Real& u6p, Real& uxp,
                                           Real& rfp, MsCounts& n) {
    // torque on the neighbour of the force fs on the home site (sign sg) at its site offset db, plus tb
    auto jtorque = [&](const Real* fs, Real sg, const Real* db, const Real* tb) {
        if (!N3) return;
        mq[0] += sg * (fs[1] * db[2] - fs[2] * db[1]);
        mq[1] += sg * (fs[2] * db[0] - fs[0] * db[2]);
        mq[2] += sg * (fs[0] * db[1] - fs[1] * db[0]);
        if (tb) { mq[0] += tb[0]; mq[1] += tb[1]; mq[2] += tb[2]; }
    };
    if (fl & 1) {
        const int nlb = B.nlj();
        for (int a = 0; a < A.nlj(); ++a) {
            const Real* da = da_t[a];
            const int row = (A.ljoff() + a) * A.ljtot() + B.ljoff();
            Real fa[3] = {0, 0, 0};
            for (int b = 0; b < nlb; ++b) {
                Real db[3];
                site_rec<Real>(sd + jb + MD_SITE_VEC * (uint32_t)b, db);
                const Real ds[3] = {md[0] + (da[0] - db[0]), md[1] + (da[1] - db[1]), md[2] + (da[2] - db[2])};
                const Real s2r = ds[0] * ds[0] + (ds[1] * ds[1] + ds[2] * ds[2]);
                Real f[3], Vd[3], u;
                lj_pair<Real>(ds, md, s2r, PTab<Real>::eps24(cP, row + b), PTab<Real>::sig2(cP, row + b),
                              PTab<Real>::shift6(cP, row + b), f, Vd, u);
                fa[0] += f[0]; fa[1] += f[1]; fa[2] += f[2];
                u6p += u;
                jtorque(f, (Real)1, db, nullptr);
            }
            mp[0] += da[1] * fa[2] - da[2] * fa[1];
            mp[1] += da[2] * fa[0] - da[0] * fa[2];
            mp[2] += da[0] * fa[1] - da[1] * fa[0];
            fp[0] += fa[0]; fp[1] += fa[1]; fp[2] += fa[2];
        }
        if (macro) n.lj += A.nlj() * nlb;
    }
    if (fl & 2) {
        const int b0 = B.nlj(), b1 = b0 + B.nch(), b2 = b1 + B.ndi(), b3 = B.ns();
        for (int a = A.nlj(); a < A.ns(); ++a) {
            const int ka = A.kind(a);  // warp-uniform: A is the warp's molecule
            const Real* da = da_t[a];
            const Real* ea = ea_t[a];
            const Real pa = PTab<Real>::p(cP, A.comp(), a);
            Real fa[3] = {0, 0, 0}, ta[3] = {0, 0, 0};
            Real db[3];
            auto site_j = [&](int b, Real* ds, Real* eb) {
                const uint32_t ob = jb + MD_SITE_VEC * (uint32_t)b;
                site_rec<Real>(sd + ob, db);
                site_rec<Real>(se + ob, eb);
                for (int c = 0; c < 3; ++c) ds[c] = md[c] + (da[c] - db[c]);
            };
            Real ds[3], eb[3], f[3], T[3], Tj[3], u, urf;
            if (ka == SK_CHARGE) {
                for (int b = b0; b < b1; ++b) {
                    site_j(b, ds, eb);
                    cc_body<Real>(ds, pa, PTab<Real>::p(cP, B.comp(), b), f, u);
                    for (int c = 0; c < 3; ++c) fa[c] += f[c];
                    uxp += u;
                    jtorque(f, (Real)1, db, nullptr);
                }
                for (int b = b1; b < b2; ++b) {
                    site_j(b, ds, eb);
                    cd_body<Real>(ds, pa, eb, PTab<Real>::p(cP, B.comp(), b), f, Tj, u);
                    for (int c = 0; c < 3; ++c) fa[c] += f[c];
                    uxp += u;
                    jtorque(f, (Real)1, db, Tj);
                }
                for (int b = b2; b < b3; ++b) {
                    site_j(b, ds, eb);
                    cq_body<Real>(ds, pa, eb, PTab<Real>::p(cP, B.comp(), b), f, Tj, u);
                    for (int c = 0; c < 3; ++c) fa[c] += f[c];
                    uxp += u;
                    jtorque(f, (Real)1, db, Tj);
                }
                if (macro) { n.cc += B.nch(); n.cd += B.ndi(); n.cq += B.nqu(); }
            } else if (ka == SK_DIPOLE) {
                for (int b = b0; b < b1; ++b) {
                    site_j(b, ds, eb);
                    const Real nd[3] = {-ds[0], -ds[1], -ds[2]};
                    cd_body<Real>(nd, PTab<Real>::p(cP, B.comp(), b), ea, pa, f, T, u);
                    for (int c = 0; c < 3; ++c) { fa[c] -= f[c]; ta[c] += T[c]; }
                    uxp += u;
                    jtorque(f, (Real)-1, db, nullptr);
                }
                for (int b = b1; b < b2; ++b) {
                    site_j(b, ds, eb);
                    dd_body<Real, N3>(ds, ea, pa, eb, PTab<Real>::p(cP, B.comp(), b), epsRF, f, T, u, urf, Tj);
                    for (int c = 0; c < 3; ++c) { fa[c] += f[c]; ta[c] += T[c]; }
                    uxp += u;
                    rfp += urf;
                    jtorque(f, (Real)1, db, Tj);
                }
                for (int b = b2; b < b3; ++b) {
                    site_j(b, ds, eb);
                    dq_body<Real>(ds, ea, pa, eb, PTab<Real>::p(cP, B.comp(), b), f, T, Tj, u);
                    for (int c = 0; c < 3; ++c) { fa[c] += f[c]; ta[c] += T[c]; }
                    uxp += u;
                    jtorque(f, (Real)1, db, Tj);
                }
                if (macro) { n.cd += B.nch(); n.dd += B.ndi(); n.dq += B.nqu(); }
            } else {
                for (int b = b0; b < b1; ++b) {
                    site_j(b, ds, eb);
                    const Real nd[3] = {-ds[0], -ds[1], -ds[2]};
                    cq_body<Real>(nd, PTab<Real>::p(cP, B.comp(), b), ea, pa, f, T, u);
                    for (int c = 0; c < 3; ++c) { fa[c] -= f[c]; ta[c] += T[c]; }
                    uxp += u;
                    jtorque(f, (Real)-1, db, nullptr);
                }
                for (int b = b1; b < b2; ++b) {
                    site_j(b, ds, eb);
                    const Real nd[3] = {-ds[0], -ds[1], -ds[2]};
                    dq_body<Real>(nd, eb, PTab<Real>::p(cP, B.comp(), b), ea, pa, f, Tj, T, u);
                    for (int c = 0; c < 3; ++c) { fa[c] -= f[c]; ta[c] += T[c]; }
                    uxp += u;
                    jtorque(f, (Real)-1, db, Tj);
                }
                for (int b = b2; b < b3; ++b) {
                    site_j(b, ds, eb);
                    qq_body<Real>(ds, ea, pa, eb, PTab<Real>::p(cP, B.comp(), b), f, T, Tj, u);
                    for (int c = 0; c < 3; ++c) { fa[c] += f[c]; ta[c] += T[c]; }
                    uxp += u;
                    jtorque(f, (Real)1, db, Tj);
                }
                if (macro) { n.cq += B.nch(); n.dq += B.ndi(); n.qq += B.nqu(); }
            }
            // torque of the site force about the centre plus the multipole torque
            mp[0] += (da[1] * fa[2] - da[2] * fa[1]) + ta[0];
            mp[1] += (da[2] * fa[0] - da[0] * fa[2]) + ta[1];
            mp[2] += (da[0] * fa[1] - da[1] * fa[0]) + ta[2];
            fp[0] += fa[0]; fp[1] += fa[1]; fp[2] += fa[2];
        }
    }
}

// Outputs of the multi-site kernels' Newton-3 form (md_config.pair_scheme =
// MD_PAIRS_NEWTON3): nh = the length of each row's leading part that holds
// the neighbours in higher slots (k_row_partition), and FP32 accumulators of
// the force, torque and virial that the neighbours of lower slots add to a
// molecule (cleared by k_ms_n3_store, which adds them to the state).
struct MsN3Out {
    const int* nh;
    float4 *f, *m, *v;
};

// Per-warp state of the multi-site force kernels.
template <typename Real>
struct MsWarp {
    typename Acc<Real>::type u6, ux, vir, rf;
    MsCounts n;
};

// Molecule i (the warp's, with ns sites): its site records into the warp's
// shared rows, its candidate row walked with the whole warp, every
// in-cut-off neighbour handed to `pair(neighbour component, ...)`, and
// the per-molecule sums stored.  The per-lane sums of the molecule are plain
// (a lane adds two or three molecule pairs) and combined by a compensated
// warp sum; the energy and virial sums are compensated (FP32) or plain
// (FP64) per lane over the warp's molecules.
template <typename Real, class Pair>
__device__ __forceinline__ void ms_molecule(const State& S, const float4* xlf, const Real* sd, const Real* se,
                                            uint32_t sstride, const uint32_t* nbr, const int* nnb, int maxnb,
                                            const Real (*soff)[3], uint32_t* ring, Real (*site_i)[MD_MAXS][3],
                                            int lane, int64_t i, int ns, Real epsRF, MsWarp<Real>& W, Pair pair) {
    Real pi[3];
    if (sizeof(Real) == 4) {
        const float4 p = xlf[i];
        pi[0] = p.x; pi[1] = p.y; pi[2] = p.z;
    } else {
        pi[0] = S.rx[i]; pi[1] = S.ry[i]; pi[2] = S.rz[i];
    }
    __syncwarp();
    if (lane < MD_SITE_VEC * ns && lane % MD_SITE_VEC < 3) {  // MD_SITE_VEC * MD_MAXS = 32 lanes
        site_i[0][lane / MD_SITE_VEC][lane % MD_SITE_VEC] = sd[(uint32_t)i * sstride + lane];
        site_i[1][lane / MD_SITE_VEC][lane % MD_SITE_VEC] = se[(uint32_t)i * sstride + lane];
    }
    __syncwarp();
    Real F[3] = {0, 0, 0}, M[3] = {0, 0, 0}, V[3] = {0, 0, 0};
    auto body = [&](uint32_t e, int fl, const Real* md) {
        const uint32_t j = e & MD_INDEX_MASK;
        const bool macro = (int64_t)j > i;
        Real fp[3] = {0, 0, 0}, mp[3] = {0, 0, 0}, mq[3] = {0, 0, 0};
        Real u6p = 0, uxp = 0, rfp = 0;
        pair(S.comp[j], site_i[0], site_i[1], j * sstride, md, fl, macro, epsRF, fp, mp, mq, u6p, uxp, rfp, W.n);
        const Real vp[3] = {md[0] * fp[0], md[1] * fp[1], md[2] * fp[2]};
        for (int c = 0; c < 3; ++c) { F[c] += fp[c]; M[c] += mp[c]; V[c] += vp[c]; }
        if (macro) {
            if (fl & 2) W.n.mol += 1;
            W.u6.add(u6p);
            W.ux.add(uxp);
            W.rf.add(rfp);
            W.vir.add(vp[0] + vp[1] + vp[2]);
        }
    };
    ms_walk_row<Real>(S, xlf, soff, pi, i, nbr + (size_t)i * maxnb, nnb[i], ring, lane, body);
    const double fx = warp_total_plain(F[0]), fy = warp_total_plain(F[1]), fz = warp_total_plain(F[2]);
    const double mx = warp_total_plain(M[0]), my = warp_total_plain(M[1]), mz = warp_total_plain(M[2]);
    const double vx = warp_total_plain(V[0], 0.5f), vy = warp_total_plain(V[1], 0.5f), vz = warp_total_plain(V[2], 0.5f);
    if (lane == 0) {
        S.Fx[i] = fx; S.Fy[i] = fy; S.Fz[i] = fz;
        S.Mx[i] = mx; S.My[i] = my; S.Mz[i] = mz;
        S.Vx[i] = vx; S.Vy[i] = vy; S.Vz[i] = vz;
    }
}

template <typename Real>
__device__ __forceinline__ void ms_store_partials(double* partials, int pstride, const MsWarp<Real>& W) {
    warp_partial_acc(partials, pstride, 0, W.u6, 1.f);
    warp_partial_acc(partials, pstride, 1, W.ux, 1.f);
    warp_partial_acc(partials, pstride, 2, W.vir, 1.f);
    warp_partial_acc(partials, pstride, 3, W.rf, -1.f);
    const int cnts[8] = {W.n.mol, W.n.lj, W.n.cc, W.n.cd, W.n.dd, W.n.cq, W.n.dq, W.n.qq};
#pragma unroll
    for (int sl = 0; sl < 8; ++sl) warp_partial_count(partials, pstride, 4 + sl, (float)cnts[sl]);
}

// The shared-memory setup common to both multi-site kernels.
#define MS_SHARED_SETUP                                                                  \
    __shared__ Real soff[27][3];                                                         \
    __shared__ uint32_t ring[MS_WARPS][128];                                             \
    __shared__ Real site_i[MS_WARPS][2][MD_MAXS][3];                                     \
    if (threadIdx.x < 27) {                                                              \
        int t = threadIdx.x;                                                             \
        soff[t][0] = (Real)((t % 3 - 1) * cP.lside[0]);                                  \
        soff[t][1] = (Real)(((t / 3) % 3 - 1) * cP.lside[1]);                            \
        soff[t][2] = (Real)((t / 9 - 1) * cP.lside[2]);                                  \
    }                                                                                    \
    __syncthreads();                                                                     \
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;                            \
    const int64_t w = (int64_t)blockIdx.x * MS_WARPS + wl;                               \
    MsWarp<Real> W;                                                                      \
    W.u6.init(); W.ux.init(); W.vir.init(); W.rf.init();                                 \
    const Real epsRF = (Real)cP.epsRFInvrc3;                                             \
    /* site records [slot][site][MD_SITE_VEC]; the host keeps cap * stride * MD_SITE_VEC < 2^32 */ \
    const uint32_t sstride = MD_SITE_VEC * (uint32_t)stride;

// The Newton-3 form of a warp's molecules base .. base + nmol - 1 (FP32).
// Each half row holds about half the in-cut-off neighbours of a full row, so
// one molecule's neighbours would leave most of its last group of 32 lanes
// idle; the ring of in-cut-off candidates therefore runs on across the warp's
// molecules, each entry tagged with its home molecule t (site records of all
// of them staged in shared memory, sites[t]: NSM sites, the most of any
// component the kernel serves), and every group of 32 lanes
// evaluates 32 molecule pairs of one or several homes.  The home's share of a
// group (F, M, m_d o F) is summed per home by a segmented warp scan (the tags
// of a group are contiguous and ascending) and added by the segment's last
// lane to the home's shared accumulator acc[t]; the neighbour's share goes to
// its global accumulators in o.  `pair(ci, cj, ...)` evaluates one molecule
// pair as in ms_molecule.
template <int NSM, class Pair>
__device__ __forceinline__ void ms_warp_n3(const State& S, const float4* xlf, const float* sd, const float* se,
                                           uint32_t sstride, const uint32_t* nbr, int maxnb,
                                           const float (*soff)[3], uint32_t* ring, float (*sites)[2][NSM][3],
                                           float (*acc)[9], int lane, int64_t base, int nmol, float epsRF,
                                           MsWarp<float>& W, MsN3Out o, Pair pair) {
    const unsigned FULL = 0xffffffffu;
    // site records and accumulators of the warp's molecules
    __syncwarp();
    for (uint32_t k = lane; k < (uint32_t)nmol * sstride; k += 32) {
        const uint32_t t = k / sstride, r = k % sstride, a = r / MD_SITE_VEC, c = r % MD_SITE_VEC;
        if (c < 3 && a < NSM) {
            sites[t][0][a][c] = sd[(uint32_t)base * sstride + k];
            sites[t][1][a][c] = se[(uint32_t)base * sstride + k];
        }
    }
    for (int k = lane; k < 32 * 9; k += 32) acc[k / 9][k % 9] = 0.f;
    __syncwarp();
    int head = 0, qn = 0;
    const unsigned lt = (1u << lane) - 1u;
    // one group: the ring's next nl entries, one per lane
    auto group = [&](int nl) {
        const int p = (head + lane) & 63;
        const uint32_t e = ring[p], tf = ring[64 + p];
        __syncwarp();
        head = (head + nl) & 63;
        qn -= nl;
        const bool act = lane < nl;
        const int t = act ? (int)(tf >> 2) : 32 + lane;  // idle lanes: tags of their own above every home's
        float v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (act) {
            const int64_t i = base + t;
            const uint32_t j = e & MD_INDEX_MASK;
            const float4 p4 = xlf[i];
            const float pi[3] = {p4.x, p4.y, p4.z};
            float md[3];
            ms_centre_distance<float>(S, xlf, soff, pi, i, e, md);
            float fp[3] = {0, 0, 0}, mp[3] = {0, 0, 0}, mq[3] = {0, 0, 0};
            float u6p = 0, uxp = 0, rfp = 0;
            const bool macro = (int64_t)j > i;  // always: the half rows hold higher slots only
            pair(S.comp[i], S.comp[j], sites[t][0], sites[t][1], j * sstride, md, (int)(tf & 3u), macro, epsRF, fp,
                 mp, mq, u6p, uxp, rfp, W.n);
            const float vp[3] = {md[0] * fp[0], md[1] * fp[1], md[2] * fp[2]};
            if (macro) {
                if (tf & 2u) W.n.mol += 1;
                W.u6.add(u6p);
                W.ux.add(uxp);
                W.rf.add(rfp);
                W.vir.add(vp[0] + vp[1] + vp[2]);
            }
            atomicAdd(&o.f[j], make_float4(-fp[0], -fp[1], -fp[2], 0.f));
            atomicAdd(&o.m[j], make_float4(mq[0], mq[1], mq[2], 0.f));
            atomicAdd(&o.v[j], make_float4(0.5f * vp[0], 0.5f * vp[1], 0.5f * vp[2], 0.f));
            for (int c = 0; c < 3; ++c) { v[c] = fp[c]; v[3 + c] = mp[c]; v[6 + c] = vp[c]; }
        }
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int tu = __shfl_up_sync(FULL, t, off);
            const bool same = lane >= off && tu == t;
#pragma unroll
            for (int c = 0; c < 9; ++c) {
                const float u = __shfl_up_sync(FULL, v[c], off);
                if (same) v[c] += u;
            }
        }
        const int tn = __shfl_down_sync(FULL, t, 1);
        if (act && (lane == 31 || tn != t)) {  // last lane of its home's segment (distinct homes)
#pragma unroll
            for (int c = 0; c < 9; ++c) acc[t][c] += v[c];
        }
        __syncwarp();
    };
    for (int t = 0; t < nmol; ++t) {
        const int64_t i = base + t;
        const float4 p4 = xlf[i];
        const float pi[3] = {p4.x, p4.y, p4.z};
        const uint32_t* row = nbr + (size_t)i * maxnb;
        const int cnt = o.nh[i];
        for (int k0 = 0; k0 < cnt; k0 += 32) {
            const int k = k0 + lane;
            int fl = 0;
            uint32_t e = 0u;
            if (k < cnt) {
                e = __ldg(&row[k]);
                float md[3];
                ms_centre_distance<float>(S, xlf, soff, pi, i, e, md);
                fl = ms_flags<float>(S, i, e, md);
            }
            const unsigned bal = __ballot_sync(FULL, fl != 0);
            if (fl) {
                const int q = (head + qn + __popc(bal & lt)) & 63;
                ring[q] = e;
                ring[64 + q] = (uint32_t)fl | ((uint32_t)t << 2);
            }
            qn += __popc(bal);
            __syncwarp();
            if (qn >= 32) group(32);
        }
    }
    if (qn > 0) group(qn);
    // the homes' sums into the state (the neighbours' shares follow in k_ms_n3_store)
    if (lane < nmol) {
        const int64_t i = base + lane;
        const float* a = acc[lane];
        S.Fx[i] = f2d_exact(a[0]); S.Fy[i] = f2d_exact(a[1]); S.Fz[i] = f2d_exact(a[2]);
        S.Mx[i] = f2d_exact(a[3]); S.My[i] = f2d_exact(a[4]); S.Mz[i] = f2d_exact(a[5]);
        S.Vx[i] = f2d_exact(0.5f * a[6]); S.Vy[i] = f2d_exact(0.5f * a[7]); S.Vz[i] = f2d_exact(0.5f * a[8]);
    }
    __syncwarp();
}

// General multi-site molecules: all site pairs of every molecule pair inside
// the molecule-centre cut-off (rc_lj for LJ centres, rc for the multipoles),
// with calcFM folded in: F = sum f, M = sum d_site x f + multipole torques,
// Vi = 1/2 sum m_d o f.  One warp per molecule, 32 molecules per warp one
// after another; component signatures read at run time.
template <typename Real, bool N3 = false>
__global__ void __launch_bounds__(MS_WARPS * 32, sizeof(Real) == 4 ? (N3 ? MS_N3_MIN_BLOCKS : MS_MIN_BLOCKS) : 3) k_force_ms(State S, const float4* xlf, const Real* sd, const Real* se,
                                                            int stride, const uint32_t* nbr, const int* nnb, int maxnb,
                                                            double* partials, int pstride, MsN3Out o) {
    MS_SHARED_SETUP
    if constexpr (N3) {
        __shared__ float sites[MS_WARPS][MS_MOLS][2][MD_MAXS][3];
        __shared__ float acc[MS_WARPS][MS_MOLS][9];
        const int64_t base = w * MS_MOLS;
        const int nmol = (int)min((int64_t)MS_MOLS, S.n - base);
        if (nmol > 0) {  // warp-uniform
            auto pair = [&](int ci, int cj, const float (*da_t)[3], const float (*ea_t)[3], uint32_t jb, const float* md,
                            int fl, bool macro, float eps, float* fp, float* mp, float* mq, float& u6p, float& uxp,
                            float& rfp, MsCounts& n) {
                const SigDyn A{cP.comp[ci], ci}, B{cP.comp[cj], cj};
                ms_molpair<float, true>(A, B, da_t, ea_t, sd, se, jb, md, fl, macro, eps, fp, mp, mq, u6p, uxp, rfp, n);
            };
            ms_warp_n3<MD_MAXS>(S, xlf, sd, se, sstride, nbr, maxnb, soff, ring[wl], sites[wl], acc[wl], lane, base, nmol,
                       epsRF, W, o, pair);
        }
    } else {
        for (int t = 0; t < MS_MOLS; ++t) {
            const int64_t i = w * MS_MOLS + t;
            if (i >= S.n) break;  // warp-uniform
            const int ci = S.comp[i];
            const SigDyn A{cP.comp[ci], ci};
            auto pair = [&](int cj, const Real (*da_t)[3], const Real (*ea_t)[3], uint32_t jb, const Real* md, int fl,
                            bool macro, Real eps, Real* fp, Real* mp, Real* mq, Real& u6p, Real& uxp, Real& rfp,
                            MsCounts& n) {
                const SigDyn B{cP.comp[cj], cj};
                ms_molpair<Real>(A, B, da_t, ea_t, sd, se, jb, md, fl, macro, eps, fp, mp, mq, u6p, uxp, rfp, n);
            };
            ms_molecule<Real>(S, xlf, sd, se, sstride, nbr, nnb, maxnb, soff, ring[wl], site_i[wl], lane, i, A.ns(),
                              epsRF, W, pair);
        }
    }
    ms_store_partials<Real>(partials, pstride, W);
}

// The same for a two-component system whose component signatures are S0 and
// S1 at compile time (chosen at setup when the components match a compiled
// pair of signatures): every molecule pair's site loops are straight code.
template <typename Real, class S0, class S1, bool N3 = false>
__global__ void __launch_bounds__(MS_WARPS * 32, sizeof(Real) == 4 ? (N3 ? MS2_N3_MIN_BLOCKS : MS_MIN_BLOCKS) : 3) k_force_ms2(State S, const float4* xlf, const Real* sd, const Real* se,
                                                             int stride, const uint32_t* nbr, const int* nnb, int maxnb,
                                                             double* partials, int pstride, MsN3Out o) {
    MS_SHARED_SETUP
    if constexpr (N3) {
        constexpr int NSM = S0::ns() > S1::ns() ? S0::ns() : S1::ns();
        __shared__ float sites[MS_WARPS][MS_MOLS][2][NSM][3];
        __shared__ float acc[MS_WARPS][MS_MOLS][9];
        const int64_t base = w * MS_MOLS;
        const int nmol = (int)min((int64_t)MS_MOLS, S.n - base);
        if (nmol > 0) {  // warp-uniform
            auto pair = [&](int ci, int cj, const float (*da_t)[3], const float (*ea_t)[3], uint32_t jb, const float* md,
                            int fl, bool macro, float eps, float* fp, float* mp, float* mq, float& u6p, float& uxp,
                            float& rfp, MsCounts& n) {
                DispFix2<S0, S1>::run(ci, [&](auto A) {
                    DispFix2<S0, S1>::run(cj, [&](auto B) {
                        ms_molpair<float, true>(A, B, da_t, ea_t, sd, se, jb, md, fl, macro, eps, fp, mp, mq, u6p, uxp,
                                                rfp, n);
                    });
                });
            };
            ms_warp_n3<NSM>(S, xlf, sd, se, sstride, nbr, maxnb, soff, ring[wl], sites[wl], acc[wl], lane, base, nmol,
                       epsRF, W, o, pair);
        }
    } else {
        for (int t = 0; t < MS_MOLS; ++t) {
            const int64_t i = w * MS_MOLS + t;
            if (i >= S.n) break;  // warp-uniform
            const int ci = S.comp[i];
            // one instance of the site-pair code per (home, neighbour) signature pair; the molecule-level code
            // around it exists once
            auto pair = [&](int cj, const Real (*da_t)[3], const Real (*ea_t)[3], uint32_t jb, const Real* md, int fl,
                            bool macro, Real eps, Real* fp, Real* mp, Real* mq, Real& u6p, Real& uxp, Real& rfp,
                            MsCounts& n) {
                DispFix2<S0, S1>::run(ci, [&](auto A) {
                    DispFix2<S0, S1>::run(cj, [&](auto B) {
                        ms_molpair<Real>(A, B, da_t, ea_t, sd, se, jb, md, fl, macro, eps, fp, mp, mq, u6p, uxp, rfp,
                                         n);
                    });
                });
            };
            ms_molecule<Real>(S, xlf, sd, se, sstride, nbr, nnb, maxnb, soff, ring[wl], site_i[wl], lane, i,
                              cP.comp[ci].ns, epsRF, W, pair);
        }
    }
    ms_store_partials<Real>(partials, pstride, W);
}

// The Newton-3 form's accumulators added to the per-molecule outputs the pair
// kernel stored (F, M, Vi of the molecule's own row) and cleared: FP32 values
// converted exactly and added in FP64.
__global__ void k_ms_n3_store(State S, MsN3Out o) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 a = o.f[i], b = o.m[i], c = o.v[i];
    o.f[i] = z; o.m[i] = z; o.v[i] = z;
    S.Fx[i] += f2d_exact(a.x); S.Fy[i] += f2d_exact(a.y); S.Fz[i] += f2d_exact(a.z);
    S.Mx[i] += f2d_exact(b.x); S.My[i] += f2d_exact(b.y); S.Mz[i] += f2d_exact(b.z);
    S.Vx[i] += f2d_exact(c.x); S.Vy[i] += f2d_exact(c.y); S.Vz[i] += f2d_exact(c.z);
}

// Signatures the two-component kernel is compiled for: the 2CLJQ + 1CLJD
// mixture (two LJ centres and a quadrupole; one LJ centre and a dipole).
typedef SigFix<0, 2, 0, 0, 1, 0, 3> SigMixA;
typedef SigFix<1, 1, 0, 1, 0, 2, 3> SigMixB;

// ------------------------------------------------------------------ integration
// FullMolecule::upd_preF; afterwards the FP32 local coordinates and the
// displacement since the last list build (for the rebuild test).
// The positions are written to rxo/ryo/rzo (the state's own arrays, or the
// other position buffer of md_run's fused steps).
__global__ void k_pre(State S, Kick K, float4* xlf, const double* origin, const float4* xlref, unsigned* disp_max,
                      double* rxo, double* ryo, double* rzo) {
    __shared__ float smax[8];
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < S.n) {
        const int ci = S.comp[i];
        const CompDev& C = cP.comp[ci];
        const double dt = K.dt, dt_halve = K.dt_halve;
        const double dtInv2m = kick_dtInv2m(K, ci);
        double vx = S.vx[i] + dtInv2m * S.Fx[i];
        double vy = S.vy[i] + dtInv2m * S.Fy[i];
        double vz = S.vz[i] + dtInv2m * S.Fz[i];
        double rx = S.rx[i] + dt * vx, ry = S.ry[i] + dt * vy, rz = S.rz[i] + dt * vz;
        S.vx[i] = vx; S.vy[i] = vy; S.vz[i] = vz;
        rxo[i] = rx; ryo[i] = ry; rzo[i] = rz;
        if (!C.skip_rot) {
            double q[4] = {S.qw[i], S.qx[i], S.qy[i], S.qz[i]};
            double L[3] = {S.Lx[i], S.Ly[i], S.Lz[i]};
            double w[3];
            // q is a unit quaternion here (normalised at the end of the last step and by k_sites), as is qh below
            qrotinv_unit(q[0], q[1], q[2], q[3], L, w);
            for (int d = 0; d < 3; ++d) w[d] *= C.invI[d];
            double qh[4];
            qh[0] = .5 * (-q[1] * w[0] - q[2] * w[1] - q[3] * w[2]);
            qh[1] = .5 * (q[0] * w[0] - q[3] * w[1] + q[2] * w[2]);
            qh[2] = .5 * (q[3] * w[0] + q[0] * w[1] - q[1] * w[2]);
            qh[3] = .5 * (-q[2] * w[0] + q[1] * w[1] + q[0] * w[2]);
            for (int e = 0; e < 4; ++e) qh[e] = qh[e] * dt_halve + q[e];
            double qc = rsqrt(qh[0] * qh[0] + qh[1] * qh[1] + qh[2] * qh[2] + qh[3] * qh[3]);  // as in k_sites
            for (int e = 0; e < 4; ++e) qh[e] *= qc;
            L[0] += dt_halve * S.Mx[i]; L[1] += dt_halve * S.My[i]; L[2] += dt_halve * S.Mz[i];
            qrotinv_unit(qh[0], qh[1], qh[2], qh[3], L, w);
            for (int d = 0; d < 3; ++d) w[d] *= C.invI[d];
            double qi[4];
            qi[0] = .5 * (-qh[1] * w[0] - qh[2] * w[1] - qh[3] * w[2]);
            qi[1] = .5 * (qh[0] * w[0] - qh[3] * w[1] + qh[2] * w[2]);
            qi[2] = .5 * (qh[3] * w[0] + qh[0] * w[1] - qh[1] * w[2]);
            qi[3] = .5 * (-qh[2] * w[0] + qh[1] * w[1] + qh[0] * w[2]);
            for (int e = 0; e < 4; ++e) q[e] += qi[e] * dt;
            qc = rsqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
            for (int e = 0; e < 4; ++e) q[e] *= qc;
            S.qw[i] = q[0]; S.qx[i] = q[1]; S.qy[i] = q[2]; S.qz[i] = q[3];
            S.Lx[i] = L[0]; S.Ly[i] = L[1]; S.Lz[i] = L[2];
        }
        float4 p;
        p.x = d2f_int(rx - origin[3 * i]);
        p.y = d2f_int(ry - origin[3 * i + 1]);
        p.z = d2f_int(rz - origin[3 * i + 2]);
        const float4 q0 = xlref[i];
        p.w = q0.w;
        xlf[i] = p;
        const float ddx = p.x - q0.x, ddy = p.y - q0.y, ddz = p.z - q0.z;
        d2 = ddx * ddx + ddy * ddy + ddz * ddz;
    }
    for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, o));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = d2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, smax[w]);
        atomicMax(disp_max, __float_as_uint(m));
    }
}

// Reduced memory mode, PositionCellProcessorRMM::processCell
// (PositionCellProcessorRMM.h:33-60): r += dt v for every molecule, nothing
// else (written to rxo/ryo/rzo: the state's own arrays, or the other position
// buffer of md_rmm_run's fused steps); then the FP32 local coordinates and the
// displacement since the last list build, as in k_pre.
__global__ void k_rmm_drift(State S, double dt, float4* xlf, const double* origin, const float4* xlref,
                            unsigned* disp_max, double* rxo, double* ryo, double* rzo) {
    __shared__ float smax[8];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < S.n) {
        const double rx = S.rx[i] + dt * S.vx[i], ry = S.ry[i] + dt * S.vy[i], rz = S.rz[i] + dt * S.vz[i];
        rxo[i] = rx; ryo[i] = ry; rzo[i] = rz;
        const float4 q0 = xlref[i];
        float4 p;
        p.x = d2f_int(rx - origin[3 * i]);
        p.y = d2f_int(ry - origin[3 * i + 1]);
        p.z = d2f_int(rz - origin[3 * i + 2]);
        p.w = q0.w;
        xlf[i] = p;
        const float ddx = p.x - q0.x, ddy = p.y - q0.y, ddz = p.z - q0.z;
        d2 = ddx * ddx + ddy * ddy + ddz * ddz;
    }
    for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, o));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = d2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, smax[w]);
        atomicMax(disp_max, __float_as_uint(m));
    }
}

// VelocityCellProcessorRMM::processCell (VelocityCellProcessorRMM.h:95-128):
// sum v.v over all molecules (no mass) into slot 12.
__global__ void k_rmm_vsum(State S, double* partials, int pstride) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double v2 = 0.0;
    if (i < S.n) v2 = rmm_v2(S.vx[i], S.vy[i], S.vz[i]);
    warp_partial(partials, pstride, 12, v2);
}

// Copy of the three position arrays (the rebuilt master state into the
// other position buffer of md_run's fused steps).
__global__ void k_copy_r(const double* ax, const double* ay, const double* az, double* bx, double* by, double* bz,
                         int64_t n, const unsigned* need) {
    if (need && !*need) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bx[i] = ax[i];
        by[i] = ay[i];
        bz[i] = az[i];
    }
}

// Rebuild when two molecules may have approached by more than the skin.
// Inside a captured graph the decision also sets the condition of the IF
// node that holds the rebuild kernels (cond != 0), so a step without a
// rebuild launches none of them.
__global__ void k_check_rebuild(unsigned* disp_max, unsigned* need, float half_skin2, int force,
                                unsigned long long* nrebuild, cudaGraphConditionalHandle cond) {
    float m = __uint_as_float(*disp_max);
    const unsigned go = (force || m > half_skin2) ? 1u : 0u;
    *need = go;
    if (go) {
        *disp_max = 0u;
        *nrebuild += 1ull;
    }
    if (cond) cudaGraphSetConditional(cond, go);
}

__global__ void k_sum_int(const int* a, int64_t n, unsigned long long* out) {
    unsigned long long s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)a[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// FullMolecule::upd_postF with the Leapfrog sums.
// With MIXED the rotational energy I w^2 (an observable: the state update is
// FP64 either way) comes from an FP32 w = I^-1 R(q)^T L, as the fused
// single-centre steps form their kinetic terms in FP32.
template <bool MIXED>
__global__ void k_post(State S, Kick K, double* partials, int pstride, int percomp) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double mv2 = 0.0, iw2 = 0.0;
    if (i < S.n) {
        const int ci = S.comp[i];
        const CompDev& C = cP.comp[ci];
        const double dt_halve = K.dt_halve;
        const double dtInv2m = kick_dtInv2m(K, ci);
        double v[3] = {S.vx[i], S.vy[i], S.vz[i]};
        double F[3] = {S.Fx[i], S.Fy[i], S.Fz[i]};
        double v2 = 0.;
        for (int d = 0; d < 3; ++d) {
            v[d] += dtInv2m * F[d];
            v2 += v[d] * v[d];
        }
        mv2 = C.m * v2;
        S.vx[i] = v[0]; S.vy[i] = v[1]; S.vz[i] = v[2];
        if (!C.skip_rot) {  // L and M are only read for molecules that rotate
            double L[3] = {S.Lx[i] + dt_halve * S.Mx[i], S.Ly[i] + dt_halve * S.My[i], S.Lz[i] + dt_halve * S.Mz[i]};
            S.Lx[i] = L[0]; S.Ly[i] = L[1]; S.Lz[i] = L[2];
            if (MIXED) {
                const float Lf[3] = {d2f_int(L[0]), d2f_int(L[1]), d2f_int(L[2])};
                float w[3], e = 0.f;
                qrotinvf(d2f_int(S.qw[i]), d2f_int(S.qx[i]), d2f_int(S.qy[i]), d2f_int(S.qz[i]), Lf, w);
                for (int d = 0; d < 3; ++d) {
                    w[d] *= C.invIf[d];
                    e += C.If[d] * w[d] * w[d];
                }
                iw2 = f2d_exact(e);
            } else {
                double w[3];
                qrotinv(S.qw[i], S.qx[i], S.qy[i], S.qz[i], L, w);
                for (int d = 0; d < 3; ++d) {
                    w[d] *= C.invI[d];
                    iw2 += C.I[d] * w[d] * w[d];
                }
            }
        }
    }
    warp_partial(partials, pstride, 12, mv2);
    if (cP.any_rotation) warp_partial(partials, pstride, 13, iw2);
    if (percomp) {  // per-component sums for component-wise thermostats
        const int c = i < S.n ? S.comp[i] : -1;
        for (int q = 0; q < percomp; ++q) {
            warp_partial(partials, pstride, SLOT_MV2_C + q, c == q ? mv2 : 0.0);
            warp_partial(partials, pstride, SLOT_IW2_C + q, c == q ? iw2 : 0.0);
        }
    }
}

// upd_postF of step k fused with upd_preF of step k + 1 for systems where no
// molecule rotates (both half kicks use the same F): the same FP64
// operations in the same order as k_post followed by k_pre, one pass over
// the state instead of two.
// With MIXED the kinetic-energy terms m v^2 are FP32 products of the
// rounded velocities, summed per warp with compensation (FP64 from there on,
// like the other global sums); the state update itself is FP64 either way.
template <bool MIXED>
__global__ void k_post_pre(State S, Kick K, double* partials, int pstride, float4* xlf, const double* origin,
                           const float4* xlref, unsigned* disp_max) {
    __shared__ float smax[8];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double mv2 = 0.0;
    float mv2f = 0.f;
    float d2 = 0.f;
    if (i < S.n) {
        const int ci = S.comp[i];
        const CompDev& C = cP.comp[ci];
        const double dt = K.dt;
        const double dtInv2m = kick_dtInv2m(K, ci);
        const double F[3] = {S.Fx[i], S.Fy[i], S.Fz[i]};
        double v[3] = {S.vx[i], S.vy[i], S.vz[i]};
        for (int d = 0; d < 3; ++d) v[d] += dtInv2m * F[d];
        if (MIXED) {
            const float vx = d2f_int(v[0]), vy = d2f_int(v[1]), vz = d2f_int(v[2]);
            mv2f = kick_massf(K, ci) * (vx * vx + (vy * vy + vz * vz));
        } else {
            double v2 = 0.;
            for (int d = 0; d < 3; ++d) v2 += v[d] * v[d];
            mv2 = C.m * v2;
        }
        for (int d = 0; d < 3; ++d) v[d] = v[d] + dtInv2m * F[d];
        const double rx = S.rx[i] + dt * v[0], ry = S.ry[i] + dt * v[1], rz = S.rz[i] + dt * v[2];
        S.vx[i] = v[0]; S.vy[i] = v[1]; S.vz[i] = v[2];
        S.rx[i] = rx; S.ry[i] = ry; S.rz[i] = rz;
        const float4 q0 = xlref[i];
        float4 p;
        p.x = d2f_int(rx - origin[3 * i]);
        p.y = d2f_int(ry - origin[3 * i + 1]);
        p.z = d2f_int(rz - origin[3 * i + 2]);
        p.w = q0.w;
        xlf[i] = p;
        const float ddx = p.x - q0.x, ddy = p.y - q0.y, ddz = p.z - q0.z;
        d2 = ddx * ddx + ddy * ddy + ddz * ddz;
    }
    if (MIXED) warp_partial_f32(partials, pstride, 12, mv2f);
    else warp_partial(partials, pstride, 12, mv2);
    for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_down_sync(0xffffffffu, d2, o));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = d2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, smax[w]);
        atomicMax(disp_max, __float_as_uint(m));
    }
}

#include "md_n3.inc"
#include "md_adjoint.inc"
#include "md_api.inc"
#include "md_planar.inc"
#include "md_tempctl.inc"
#include "md_batch.inc"
