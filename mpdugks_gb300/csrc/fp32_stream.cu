// FP32 deviation-storage DUGKS step, streaming form, single case: the kernel
// k_stream32 over the (strip, row segment) items of one grid, its launcher, and the
// tensor map of its TMA row loads.  What a warp does per item is stream_item
// (fp32_stream.cuh), shared with the batched serving kernel.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

// constants, ring layouts, TMA helpers shared with the batched streaming kernel
#include "fp32_stream.cuh"

namespace dugks {
namespace f32 {

// first: the first step after an initialisation (the collision takes the state the
// initialisation left instead of the macroscopic quantities of the deviations).  A
// runtime flag, as in the tile kernels, so that both compile the per-cell stages alike
// (the same multiply-add contractions) and give bit-identical results.
// TMA: the stage ring is filled by TMA row loads from `tmap`, a 3-D map (columns,
// rows, planes) over both state copies, the copy a step reads starting at plane
// zin; strips whose window wraps around the periodic x boundary, and slab
// partitions, load per lane with cp.async.  A load not complete within
// TMA_WAIT_LIMIT polls sets *err and ends the warp.
// The per-item work is stream_item (fp32_stream.cuh), the same function the batched
// serving kernel runs, so a change to the steps lands in both.
template <int MODEL, bool WALLS, bool TMA, bool NEE>
__global__ void __launch_bounds__(WPB * 32, STREAM_MIN_BLOCKS)
    k_stream32(P32 P, S32 S, int first, int gin, int gout, uint32_t step, int nstrips, int nsegs, int seg_rows,
               const __grid_constant__ CUtensorMap tmap, int zin, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *wbase = reinterpret_cast<float *>(smem_raw) + (size_t)wib * WARP_F;
    float *stg = wbase;                   // [NSTG][STG_PLANES][32]
    float *bring = wbase + STG_F;         // [3] row slots
    float *aring = wbase + STG_F + BR_F;  // [3] row slots
    // mbarriers of this warp's stage slots; their phase parities (bit s: slot s)
    const unsigned bar0 = smem_u32(smem_raw + (size_t)WPB * WARP_F * sizeof(float) + (size_t)wib * NSTG * 8);
    const bool tma_ok = TMA && (smem_u32(smem_raw) & 127u) == 0 && !(P.halo_lo || P.halo_hi);
    uint32_t phases = 0;
    if (TMA) {
        if (lane == 0) {
#pragma unroll
            for (int s = 0; s < NSTG; ++s) mbar_init(bar0 + 8 * s);
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        __syncwarp();
    }
    const int ny = P.ny;
    const int gw = blockIdx.x * WPB + wib, nw = gridDim.x * WPB;
    for (int item = gw; item < nstrips * nsegs; item += nw) {
        const int strip = item % nstrips, seg = item / nstrips;
        const int y0 = seg * seg_rows, y1 = min(y0 + seg_rows, ny);
        if (!stream_item<MODEL, WALLS, TMA, NEE>(P, S, first, gin, gout, step, strip, y0, y1, tma_ok, &tmap, zin, err, stg,
                                            bring, aring, bar0, phases, lane))
            return;
    }
}

static int g_stream_nsm = 0, g_stream_blocks = 0;

// Rows of a strip segment.  The persistent warps take the (strip, segment) items in
// turn, so a step lasts as long as the warps with the most items.  First choice: the
// longest of 128, 64, 32 rows that still gives every resident warp about 4 items (a long
// segment costs fewer warm-up rows).  Where that leaves fewer than 8 rounds of items,
// the last, partly filled round is a large share of the step (measured: 2048^2 in 32-row
// segments, 1.3 rounds, takes 1.28x the time of the best length), and the length is
// searched instead: the fill of the last round, (items / warps) / ceil(items / warps),
// times the share of a segment that is not warm-up, len / (len + 4), is maximised.
int stream_segment_rows(int nstrips, int ny, int warps) {
    int seg = SEG_MAX;
    while (seg > 32 && (long long)nstrips * ((ny + seg - 1) / seg) < 4LL * warps) seg /= 2;
    if ((double)nstrips * ((ny + seg - 1) / seg) >= 8.0 * warps) return seg;
    int best = seg;
    double best_eff = -1.0;
    for (int len = 16; len <= ny; ++len) {
        const int n = (ny + len - 1) / len;
        const double waves = (double)nstrips * n / warps;
        const double eff = waves / std::ceil(waves) * ((double)ny / n / ((double)ny / n + 4.0));
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = len;
        }
    }
    return best;
}

template <int MODEL, bool WALLS, bool TMA, bool NEE>
static cudaError_t stream_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_stream32<MODEL, WALLS, TMA, NEE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STREAM_SMEM);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stream32<MODEL, WALLS, TMA, NEE>, WPB * 32,
                                                      STREAM_SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    g_stream_blocks = g_stream_blocks ? min(g_stream_blocks, per_sm) : per_sm;
    return cudaSuccess;
}

template <int MODEL, bool WALLS, bool NEE>
static cudaError_t launch_stream_t(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                                   uint32_t step, const CUtensorMap *tmap, int zin, int *err, bool *fallback) {
    static bool ready = false;
    if (!ready) {
        cudaError_t e = stream_prepare<MODEL, WALLS, false, NEE>();
        if (e != cudaSuccess) return e;
        if ((e = stream_prepare<MODEL, WALLS, true, NEE>()) != cudaSuccess) return e;
        int dev = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&g_stream_nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        ready = true;
    }
    // the longest segment that still gives every resident warp about 4 segments
    // (a long segment costs fewer warm-up rows, a short one less idle tail)
    const int nstrips = (P.nx + SW - 1) / SW, warps = g_stream_nsm * g_stream_blocks * WPB;
    // a grid with fewer 32-row strip segments than a third of the resident warps leaves
    // most of the GPU idle in this form: the tile kernel (same arithmetic, same results)
    // runs it.  Measured (Rayleigh-Taylor, G cell-updates/s, streaming / tile): 256x1024
    // 5.1 / 7.5 (320 segments), 768^2 9.2 / 8.5 (672), 512x2048 11.9 / 8.5 (1216), 1024^2
    // 12.5 / 8.8 (1184), against 1824 resident warps.  (A slab partition reads halo rows,
    // which only this form does, and so do NEE walls: it always runs those.)
    if (!NEE && !(P.halo_lo || P.halo_hi) && 3LL * nstrips * ((P.ny + 31) / 32) < warps) {
        *fallback = true;
        return cudaSuccess;
    }
    const int seg = stream_segment_rows(nstrips, P.ny, warps);
    const int nsegs = (P.ny + seg - 1) / seg;
    const int items = nstrips * nsegs;
    const int blocks = min((items + WPB - 1) / WPB, g_stream_nsm * g_stream_blocks);
    if (tmap) {
        k_stream32<MODEL, WALLS, true, NEE><<<blocks, WPB * 32, STREAM_SMEM, st>>>(P, S, first, gin, gout, step,
                                                                                 nstrips, nsegs, seg, *tmap, zin, err);
    } else {
        CUtensorMap none;
        memset(&none, 0, sizeof none);
        k_stream32<MODEL, WALLS, false, NEE><<<blocks, WPB * 32, STREAM_SMEM, st>>>(P, S, first, gin, gout, step,
                                                                                  nstrips, nsegs, seg, none, 0, err);
    }
    return cudaGetLastError();
}

cudaError_t launch_step32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                          int64_t *launches, uint32_t step);

// tmap: null, or the handle's 3-D tensor map over its two state copies (stream_tensor_map);
// zin: the first plane of the copy this step reads (0 or PL_N); err: the word a staged
// load that did not complete sets
cudaError_t launch_stream32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                            int64_t *launches, uint32_t step, const void *tmap, int zin, int *err) {
    // the row window of a segment wraps at most once: grids of fewer than 8 rows
    // run the tile kernel (same arithmetic, same results)
    if (P.ny < 8) return launch_step32(P, S, first, gin, gout, st, launches, step);
    const CUtensorMap *tm = static_cast<const CUtensorMap *>(tmap);
    cudaError_t e = cudaErrorInvalidValue;
    bool fallback = false;
    // NEE walls run the streaming form (the tile kernel has bounce-back walls only)
    switch (P.model * 4 + (P.walls ? 2 : 0) + (P.walls && P.nee ? 1 : 0)) {
        case AC * 4 + 0:
            e = launch_stream_t<AC, false, false>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        case AC * 4 + 2:
            e = launch_stream_t<AC, true, false>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        case AC * 4 + 3:
            e = launch_stream_t<AC, true, true>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        case HCZ * 4 + 0:
            e = launch_stream_t<HCZ, false, false>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        case HCZ * 4 + 2:
            e = launch_stream_t<HCZ, true, false>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        case HCZ * 4 + 3:
            e = launch_stream_t<HCZ, true, true>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        default: break;
    }
    if (e == cudaSuccess && fallback) return launch_step32(P, S, first, gin, gout, st, launches, step);
    if (e == cudaSuccess) *launches += 1;
    return e;
}

// A 3-D tensor map (x: nx columns, y: ny rows, z: 2 PL_N planes) over the two state
// copies of a single-case FP32 handle (PL_N planes each: 9 f, 8 g, the phi pair, 6
// aux), one plane every qs floats from `base`; box {32, 1, STG_PLANES} (the stage slot
// of one row: its f and g planes).
cudaError_t stream_tensor_map(void *map_out, float *base, int nx, int ny, int pitch, size_t qs) {
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        encode = reinterpret_cast<EncodeFn>(fn);
    }
    if (nx < 32 || ((uintptr_t)base & 15) || ((size_t)pitch * 4) % 16 || (qs * 4) % 16) return cudaErrorInvalidValue;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, 2 * PL_N};
    const cuuint64_t strides[2] = {(cuuint64_t)pitch * 4, (cuuint64_t)qs * 4};
    const cuuint32_t box[3] = {32, 1, STG_PLANES};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode(static_cast<CUtensorMap *>(map_out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims,
                              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace f32
}  // namespace dugks
