// Face and update kernels of one arithmetic form, one flow model and one
// scheme set.  Built twelve times from this file: -DHMR_FAST=0 --fmad=false
// (namespace hmr_exact_...) and -DHMR_FAST=1 (hmr_fast_...), with
// -DHMR_MODEL=0 (single species), 1 (four-equation) or 2 (five-equation), and
// -DHMR_SCHEME_SET=0 (WCNS5-JS, WCNS6-LD; namespace <form>_m<model>) or 1
// (WCNS5-Z, WCNS6-CU-M2; namespace <form>_zc_m<model>).
#include <cuda_runtime.h>

#include <type_traits>

#include "hmr_launch.h"

#ifndef HMR_MODEL
#error "HMR_MODEL must be defined: 0 single species, 1 four-equation, 2 five-equation"
#endif

#ifndef HMR_SCHEME_SET
#define HMR_SCHEME_SET 0
#endif

#define HMR_CAT2(a, b) a##b
#define HMR_CAT(a, b) HMR_CAT2(a, b)
#if HMR_FAST && HMR_SCHEME_SET
#define HMR_NS HMR_CAT(hmr_fast_zc_m, HMR_MODEL)
#elif HMR_FAST
#define HMR_NS HMR_CAT(hmr_fast_m, HMR_MODEL)
#elif HMR_SCHEME_SET
#define HMR_NS HMR_CAT(hmr_exact_zc_m, HMR_MODEL)
#else
#define HMR_NS HMR_CAT(hmr_exact_m, HMR_MODEL)
#endif

namespace HMR_NS {

using namespace hmr;

template <int D, int M, int N, int S>
struct VT {
    static constexpr int DIM = D, MODEL = M, NSP = N, SCHEME = S;
};

// Variants of this translation unit: 2D/3D x the two schemes of its set, for
// its model (one species for the single-species model, two for the
// multi-species ones).
template <class F>
static int dispatch(const Variant& v, F f) {
    constexpr int M_ = HMR_MODEL;
    constexpr int N_ = M_ == SINGLE_SPECIES ? 1 : 2;
    constexpr int S0 = HMR_SCHEME_SET ? WCNS5_Z : WCNS5_JS;
    constexpr int S1 = HMR_SCHEME_SET ? WCNS6_CU_M2 : WCNS6_LD;
    if (v.model != M_ || v.nsp != N_) return -2;
    if (v.dim == 2 && v.scheme == S0) return f(VT<2, M_, N_, S0>{});
    if (v.dim == 2 && v.scheme == S1) return f(VT<2, M_, N_, S1>{});
    if (v.dim == 3 && v.scheme == S0) return f(VT<3, M_, N_, S0>{});
    if (v.dim == 3 && v.scheme == S1) return f(VT<3, M_, N_, S1>{});
    return -2;
}

constexpr int FACE_THREADS = 128;
constexpr int UPDATE_THREADS = 128;

// The exact form computes every face; the fast form queues the faces it hands
// back (see face_item) for redo_kernel.
template <int DIM, int MODEL, int NSP, int SCHEME, int A>
__global__ void __launch_bounds__(FACE_THREADS)
faces_kernel(Params P, Geom g, Scratch S, Counters* cnt, Redo R) {
    const long nf = nface_of(g, A);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += (long)gridDim.x * blockDim.x) {
        if (face_item<!HMR_FAST, DIM, MODEL, NSP, SCHEME, A>(P, g, S, t, cnt)) redo_push(R, A, t);
    }
}

// Fast form with sorted faces: every face of axis A is classified by its sensor; the
// HLLC-HLL ones go to the exact pass's queue, the others to the axis's list, both appended a
// warp at a time (one atomic per warp and list), so a list holds runs of neighbouring faces.
template <int DIM, int A>
__global__ void __launch_bounds__(FACE_THREADS) classify_kernel(Geom g, Scratch S, Redo R) {
    const long nf = nface_of(g, A);
    const int e0 = g.n[0] + (A == 0 ? 3 : 0);
    const int e1 = g.n[1] + (A == 1 ? 3 : 0);
    const long st = (A == 0) ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
    unsigned long long* list = R.fast + R.fast_off[A];
    const unsigned lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    // blockDim.x is a multiple of 32 and every thread runs the same iterations: the warp
    // votes below see all 32 lanes
    for (long t0 = (long)blockIdx.x * blockDim.x; t0 < nf; t0 += (long)gridDim.x * blockDim.x) {
        const long t = t0 + threadIdx.x;
        const bool valid = t < nf;
        bool hll = false;
        if (valid) {
            const int i = (int)(t % e0) - (A == 0);
            const int j = (int)((t / e0) % e1) - (A == 1);
            const int k = DIM == 3 ? (int)(t / ((long)e0 * e1)) - (A == 2) : 0;
            const long xR = cidx<DIM>(g, i, j, k);
            hll = face_uses_hll(S, xR - st, xR);
        }
        const unsigned fm = __ballot_sync(0xffffffffu, valid && !hll);
        const unsigned hm = __ballot_sync(0xffffffffu, valid && hll);
        unsigned bf = 0, bh = 0;
        if (lane == 0) {
            if (fm) bf = atomicAdd(R.fast_count + A, (unsigned)__popc(fm));
            if (hm) {
                bh = atomicAdd(R.count, (unsigned)__popc(hm));
                atomicAdd(R.fast_count + 3, (unsigned)__popc(hm));
            }
        }
        bf = __shfl_sync(0xffffffffu, bf, 0);
        bh = __shfl_sync(0xffffffffu, bh, 0);
        if (valid && !hll) list[bf + __popc(fm & below)] = (unsigned long long)t;
        if (valid && hll) {
            const unsigned long long idx = bh + __popc(hm & below);
            if (idx < R.cap) R.list[idx] = ((unsigned long long)A << 56) | (unsigned long long)t;
        }
    }
}

// The exact form of one queued face, kept out of line: inlined beside the fast form, the shared
// subexpressions of the two would be merged and the fast form's multiply-add contraction (decided
// per kernel) could change, and with it its last bits against the other kernels that run it.
template <int DIM, int MODEL, int NSP, int SCHEME>
__device__ __noinline__ void exact_queued_face(const Params& P, const Geom& g, const Scratch& S, Counters* cnt,
                                               unsigned long long v) {
    const int a = (int)(v >> 56);
    const long t = (long)(v & ((1ull << 56) - 1));
    if (a == 0) face_item<true, DIM, MODEL, NSP, SCHEME, 0>(P, g, S, t, cnt);
    else if (a == 1) face_item<true, DIM, MODEL, NSP, SCHEME, 1>(P, g, S, t, cnt);
    else if constexpr (DIM == 3) face_item<true, DIM, MODEL, NSP, SCHEME, 2>(P, g, S, t, cnt);
}

// One launch over the sorted faces: the HLLC faces of every axis in the fast form (listed by
// classify_kernel), then the HLLC-HLL ones in the exact form (the first fast_count[3] entries
// of the queue).  The two sets are disjoint and each face writes its own flux, so they run side
// by side; faces the fast form hands back (first-order fallback, near a bounds threshold) are
// queued behind the HLLC-HLL ones for redo_kernel.
template <int DIM, int MODEL, int NSP, int SCHEME>
__global__ void __launch_bounds__(FACE_THREADS)
faces_sorted_kernel(Params P, Geom g, Scratch S, Counters* cnt, Redo R) {
    const long n0 = (long)R.fast_count[0];
    const long n01 = n0 + (long)R.fast_count[1];
    const long nf = n01 + (DIM == 3 ? (long)R.fast_count[2] : 0);
    const long total = nf + (long)min((unsigned long long)R.fast_count[3], R.cap);
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < total; r += (long)gridDim.x * blockDim.x) {
        if (r < n0) {
            const long t = (long)R.fast[R.fast_off[0] + r];
            if (face_item<false, DIM, MODEL, NSP, SCHEME, 0>(P, g, S, t, cnt)) redo_push(R, 0, t);
        } else if (r < n01) {
            const long t = (long)R.fast[R.fast_off[1] + (r - n0)];
            if (face_item<false, DIM, MODEL, NSP, SCHEME, 1>(P, g, S, t, cnt)) redo_push(R, 1, t);
        } else if (r < nf) {
            if constexpr (DIM == 3) {
                const long t = (long)R.fast[R.fast_off[2] + (r - n01)];
                if (face_item<false, DIM, MODEL, NSP, SCHEME, 2>(P, g, S, t, cnt)) redo_push(R, 2, t);
            }
        } else {
            exact_queued_face<DIM, MODEL, NSP, SCHEME>(P, g, S, cnt, R.list[r - nf]);
        }
    }
}

// Exact recomputation of the queued faces of one patch.
template <int DIM, int MODEL, int NSP, int SCHEME>
__global__ void __launch_bounds__(FACE_THREADS)
redo_kernel(Params P, Geom g, Scratch S, Counters* cnt, Redo R, int after_sorted) {
    const unsigned long long n = min((unsigned long long)*R.count, R.cap);
    // after faces_sorted_kernel the HLLC-HLL entries at the head of the queue are done
    const unsigned long long r0 = after_sorted ? (unsigned long long)R.fast_count[3] : 0ull;
    for (unsigned long long r = r0 + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; r < n;
         r += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long v = R.list[r];
        const int a = (int)(v >> 56);
        const long t = (long)(v & ((1ull << 56) - 1));
        if (a == 0) face_item<true, DIM, MODEL, NSP, SCHEME, 0>(P, g, S, t, cnt);
        else if (a == 1) face_item<true, DIM, MODEL, NSP, SCHEME, 1>(P, g, S, t, cnt);
        else if constexpr (DIM == 3) face_item<true, DIM, MODEL, NSP, SCHEME, 2>(P, g, S, t, cnt);
    }
}

template <int DIM, int MODEL, int NSP>
__global__ void __launch_bounds__(UPDATE_THREADS)
update_kernel(Geom g, Scratch S, UpdateArgs U) {
    const long n = ninterior_of(g);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        update_item<DIM, MODEL, NSP>(g, S, U, t);
}

static inline int grid_for(long items, int threads) {
    long b = (items + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > (1L << 30)) b = 1L << 30;
    return (int)b;
}

int launch_faces(const Variant& v, const Params& P, const Geom& g, const Scratch& S, Counters* cnt,
                 const Redo& R, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        const bool sorted = HMR_FAST && R.fast != nullptr && R.fast_count != nullptr;
        if (HMR_FAST) {
            cudaError_t e = cudaMemsetAsync(R.count, 0, sizeof(unsigned int), st);
            if (e == cudaSuccess && sorted) e = cudaMemsetAsync(R.fast_count, 0, 4 * sizeof(unsigned int), st);
            if (e != cudaSuccess) return (int)e;
        }
        if constexpr (HMR_FAST != 0) {
            if (sorted) {
                classify_kernel<T::DIM, 0><<<grid_for(nface_of(g, 0), FACE_THREADS), FACE_THREADS, 0, st>>>(g, S, R);
                classify_kernel<T::DIM, 1><<<grid_for(nface_of(g, 1), FACE_THREADS), FACE_THREADS, 0, st>>>(g, S, R);
                if constexpr (T::DIM == 3)
                    classify_kernel<T::DIM, 2><<<grid_for(nface_of(g, 2), FACE_THREADS), FACE_THREADS, 0, st>>>(g, S, R);
                long nall = 0;
                for (int a = 0; a < T::DIM; a++) nall += nface_of(g, a);
                faces_sorted_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME>
                    <<<grid_for(nall, FACE_THREADS), FACE_THREADS, 0, st>>>(P, g, S, cnt, R);
            }
        }
        if (!sorted) {
            faces_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, 0>
                <<<grid_for(nface_of(g, 0), FACE_THREADS), FACE_THREADS, 0, st>>>(P, g, S, cnt, R);
            faces_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, 1>
                <<<grid_for(nface_of(g, 1), FACE_THREADS), FACE_THREADS, 0, st>>>(P, g, S, cnt, R);
            if constexpr (T::DIM == 3)
                faces_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, 2>
                    <<<grid_for(nface_of(g, 2), FACE_THREADS), FACE_THREADS, 0, st>>>(P, g, S, cnt, R);
        }
        if (HMR_FAST) {
            int dev = 0, sms = 1;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            redo_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME><<<sms * 2, FACE_THREADS, 0, st>>>(P, g, S, cnt, R,
                                                                                            sorted ? 1 : 0);
        }
        return (int)cudaPeekAtLastError();
    });
}

int launch_update(const Variant& v, const Geom& g, const Scratch& S, const UpdateArgs& U, cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        update_kernel<T::DIM, T::MODEL, T::NSP>
            <<<grid_for(ninterior_of(g), UPDATE_THREADS), UPDATE_THREADS, 0, st>>>(g, S, U);
        return (int)cudaPeekAtLastError();
    });
}

// ---------------------------------------------------------------------------
// Batched form: one persistent kernel per RK substep over every patch of a
// level.  Phases are separated by a grid barrier; inside a phase the items of
// all patches form one flat index space that the resident blocks take in
// block-wide chunks (the small ghost phases: a grid-stride loop), so small and
// large patches share the SMs evenly.
// ---------------------------------------------------------------------------

// Grid barrier on a monotonically increasing arrival counter.  Barrier number
// b (1-based) is passed when the counter reaches b*gridDim.x.  The wait is
// bounded: after timeout_ns it raises the status flag and returns false, and
// every later barrier of the launch returns false at once, so all blocks
// leave the kernel.  `extra` > 0 makes the target unreachable (used only by
// the test that checks this give-up path).
__device__ __forceinline__ bool grid_barrier(unsigned int* counter, int* status, unsigned int b,
                                             unsigned long long timeout_ns, unsigned int extra) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(counter, 1u);
        const unsigned int target = b * (gridDim.x + extra);
        unsigned long long t0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        int ok = 1;
        while (true) {
            const unsigned int c = *((volatile unsigned int*)counter);
            if (c >= target) break;
            if (*((volatile int*)status) != 0) { ok = 0; break; }
            unsigned long long t1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
            if (t1 - t0 > timeout_ns) {
                atomicExch(status, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Patch holding flat item t of a phase (prefix offsets, binary search).
template <class OffF>
__device__ __forceinline__ int find_patch(const PatchWork* W, int np, long t, OffF off) {
    int lo = 0, hi = np - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off(W[mid]) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Items [0, total) of a phase, handed out in chunks of one block's width from a counter, in
// order: blocks that finish early take the next chunk (the order and balancing of one block
// per chunk launched on its own), and the chunks in flight stay within a narrow band of the
// index space, so that neighbouring stencil rows meet in L2 (a fixed grid-stride assignment
// lets fast and slow blocks drift apart over the phase).
// A chunk is `mult` block widths (work-splitting knob of the autotuner); a block takes its
// items in block-wide rows.
template <class F>
__device__ __forceinline__ void level_chunks(unsigned int* counter, long total, int mult, F f) {
    __shared__ unsigned int s_chunk;
    const long width = (long)blockDim.x * mult;
    const long nchunk = (total + width - 1) / width;
    while (true) {
        __syncthreads();   // every thread has read the previous chunk
        if (threadIdx.x == 0) s_chunk = atomicAdd(counter, 1u);
        __syncthreads();
        const long c = s_chunk;
        if (c >= nchunk) break;
        for (int r = 0; r < mult; r++) {
            const long t = c * width + (long)r * blockDim.x + threadIdx.x;
            if (t < total) f(t);
        }
    }
}

// The cell-wise phases (cell data, sensor, update), handed out in chunks or -- the other
// work-splitting mode -- by a fixed grid-stride assignment.
template <class F>
__device__ __forceinline__ void level_cell_items(unsigned int* counter, long total, const LevelArgs& L, F f) {
    if (L.split_mode & 1) {
        const long stride = (long)gridDim.x * blockDim.x;
        for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) f(t);
    } else {
        level_chunks(counter, total, L.chunk_mult, f);
    }
}

// Chunk counters of LevelArgs::chunk.
enum { CHUNK_FACE0 = 0, CHUNK_CELLS = 3, CHUNK_SENSOR = 4, CHUNK_UPDATE = 5, CHUNK_REDO = 6, CHUNK_SORTED = 7 };

// The level's sorting of the faces of axis A (as classify_kernel, over the level's face items):
// HLLC faces to the axis's list, HLLC-HLL faces to the head of the redo queue.  Every thread
// of the grid runs the same iterations (the warp votes see all 32 lanes).
template <int DIM, int A>
__device__ __forceinline__ void level_classify(const LevelArgs& L, const PatchWork* W, int np) {
    const long total = L.total_face[A];
    unsigned long long* list = L.sorted + L.sort_off[A];
    const unsigned lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    for (long t0 = (long)blockIdx.x * blockDim.x; t0 < total; t0 += (long)gridDim.x * blockDim.x) {
        const long t = t0 + threadIdx.x;
        const bool valid = t < total;
        bool hll = false;
        if (valid) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[A]; });
            const Geom& g = W[p].g;
            const long u = t - W[p].off_face[A];
            const int e0 = g.n[0] + (A == 0 ? 3 : 0);
            const int e1 = g.n[1] + (A == 1 ? 3 : 0);
            const int i = (int)(u % e0) - (A == 0);
            const int j = (int)((u / e0) % e1) - (A == 1);
            const int k = DIM == 3 ? (int)(u / ((long)e0 * e1)) - (A == 2) : 0;
            const long st = (A == 0) ? 1 : (A == 1 ? (long)g.G[0] : (long)g.G[0] * g.G[1]);
            const long xR = cidx<DIM>(g, i, j, k);
            hll = face_uses_hll(W[p].S, xR - st, xR);
        }
        const unsigned fm = __ballot_sync(0xffffffffu, valid && !hll);
        const unsigned hm = __ballot_sync(0xffffffffu, valid && hll);
        unsigned bf = 0, bh = 0;
        if (lane == 0) {
            if (fm) bf = atomicAdd(L.sort_count + A, (unsigned)__popc(fm));
            if (hm) {
                bh = atomicAdd(L.redo.count, (unsigned)__popc(hm));
                atomicAdd(L.sort_count + 3, (unsigned)__popc(hm));
            }
        }
        bf = __shfl_sync(0xffffffffu, bf, 0);
        bh = __shfl_sync(0xffffffffu, bh, 0);
        if (valid && !hll) list[bf + __popc(fm & below)] = (unsigned long long)t;
        if (valid && hll) {
            const unsigned long long idx = bh + __popc(hm & below);
            if (idx < L.redo.cap) L.redo.list[idx] = ((unsigned long long)A << 56) | (unsigned long long)t;
        }
    }
}

// The exact form of one queued level face, out of line (see exact_queued_face).
template <int DIM, int MODEL, int NSP, int SCHEME>
__device__ __noinline__ void level_exact_face(const Params& P, const PatchWork* W, int np, unsigned long long v) {
    const int a = (int)(v >> 56);
    const long t = (long)(v & ((1ull << 56) - 1));
    if (a == 0) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[0]; });
        face_item<true, DIM, MODEL, NSP, SCHEME, 0>(P, W[p].g, W[p].S, t - W[p].off_face[0], nullptr);
    } else if (a == 1) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[1]; });
        face_item<true, DIM, MODEL, NSP, SCHEME, 1>(P, W[p].g, W[p].S, t - W[p].off_face[1], nullptr);
    } else if constexpr (DIM == 3) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[2]; });
        face_item<true, DIM, MODEL, NSP, SCHEME, 2>(P, W[p].g, W[p].S, t - W[p].off_face[2], nullptr);
    }
}

// 128 threads per block at most, with registers for three such blocks per SM (at most 170 per
// thread) in the fast form, as the per-patch face kernels use; the exact form's face item, the
// 3D multi-species models and the 3D NavierStokes phases need more registers and keep two
// blocks per SM.
constexpr int LEVEL_MAX_THREADS = 128;
template <int DIM, int MODEL, int DORD>
constexpr int level_min_blocks() {
#ifdef HMR_LEVEL_MIN_BLOCKS
    return HMR_LEVEL_MIN_BLOCKS;
#else
    return HMR_FAST && (DIM == 2 || (MODEL == SINGLE_SPECIES && DORD == 0)) ? 3 : 2;
#endif
}

// DORD: 0 for the Euler equations, 2, 4 or 6 for NavierStokes with that diffusive order (single
// species; the sixth order on 5-ghost patch arrays); a separate instantiation, so that the
// Euler kernel keeps its registers.
template <int DIM, int MODEL, int NSP, int SCHEME, int DORD>
__global__ void __launch_bounds__(LEVEL_MAX_THREADS, level_min_blocks<DIM, MODEL, DORD>())
level_kernel(Params P, LevelArgs L) {
    const long stride = (long)gridDim.x * blockDim.x;
    const long t0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const PatchWork* W = L.work;
    const int np = L.npatch;
    unsigned int b = 0;
#define HMR_BARRIER() \
    if (!grid_barrier(L.barrier, L.status, ++b, L.timeout_ns, L.barrier_extra)) return

    // Phase 0: ghost fill of the input stage: per patch (periodic, zero-gradient or provided
    // per axis), or, with a level layout, copies from neighbouring patches and periodic
    // images followed by zero-gradient at the domain's non-periodic faces.
    if (L.exchange) {
        const int sl = L.nst - 1;
        for (long t = t0; t < L.total_copy; t += stride) {
            int lo = 0, hi = L.ncopy - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (L.copies[mid].off <= t) lo = mid;
                else hi = mid - 1;
            }
            const GhostCopy& cp = L.copies[lo];
            const long u = t - cp.off;
            const int a0 = (int)(u % cp.ext[0]);
            const int a1 = (int)((u / cp.ext[0]) % cp.ext[1]);
            const int a2 = (int)(u / ((long)cp.ext[0] * cp.ext[1]));
            const PatchWork& wd = W[cp.dst];
            const PatchWork& ws = W[cp.src];
            const long xd = cidx<DIM>(wd.g, cp.dlo[0] + a0, cp.dlo[1] + a1, cp.dlo[2] + a2);
            const long xs = cidx<DIM>(ws.g, cp.slo[0] + a0, cp.slo[1] + a1, cp.slo[2] + a2);
            for (int e = 0; e < L.ncomp; e++) wd.Q[sl].p[e][xd] = ws.Q[sl].p[e][xs];
        }
        HMR_BARRIER();
        for (long t = t0; t < L.total_fill; t += stride) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_fill; });
            domain_fill_item<DIM>(W[p].g, W[p].Q[sl], L.ncomp, W[p].lo, L.dom, L.dom_periodic, t - W[p].off_fill,
                                  L.mom0, L.bvals);
        }
    } else {
        for (long t = t0; t < L.total_fill; t += stride) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_fill; });
            fill_item<DIM>(W[p].g, W[p].Q[L.nst - 1], L.ncomp, W[p].periodic, t - W[p].off_fill, L.mom0, L.bvals);
        }
    }
    HMR_BARRIER();
    level_cell_items(L.chunk + CHUNK_CELLS, L.total_cells, L, [&](long t) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_cells; });
        cells_item<DIM, MODEL, NSP>(P, W[p].g, W[p].Q[L.nst - 1], W[p].S, t - W[p].off_cells);
    });
    HMR_BARRIER();
    level_cell_items(L.chunk + CHUNK_SENSOR, L.total_sensor, L, [&](long t) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_sensor; });
        sensor_item<DIM, MODEL, NSP>(W[p].g, W[p].S, t - W[p].off_sensor);
    });
    if constexpr (DORD != 0) {
        // NavierStokes: temperature and node velocity gradient (needs the cell data only)
        for (long t = t0; t < L.total_cells; t += stride) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_cells; });
            diff_grad_item<DIM, DORD>(P, W[p].g, W[p].S, t - W[p].off_cells);
        }
    }
    HMR_BARRIER();
    if constexpr (DORD != 0) {
        // NavierStokes: midpoint diffusive fluxes (needs the node gradient), beside the faces
        for (long t = t0; t < L.total_dface[0]; t += stride) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_dface[0]; });
            diff_mid_item<DIM, DORD, 0>(P, W[p].g, W[p].S, t - W[p].off_dface[0]);
        }
        for (long t = t0; t < L.total_dface[1]; t += stride) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_dface[1]; });
            diff_mid_item<DIM, DORD, 1>(P, W[p].g, W[p].S, t - W[p].off_dface[1]);
        }
        if constexpr (DIM == 3) {
            for (long t = t0; t < L.total_dface[2]; t += stride) {
                const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_dface[2]; });
                diff_mid_item<DIM, DORD, 2>(P, W[p].g, W[p].S, t - W[p].off_dface[2]);
            }
        }
    }
    constexpr bool X = !HMR_FAST;
    unsigned long long redo_from = 0;   // queue entries before this one were done beside the fast form
    (void)redo_from;
#if HMR_FAST
    if (L.split_mode & 2) {
        // faces sorted by their sensor, then the HLLC ones in the fast form beside the
        // HLLC-HLL ones in the exact form (as faces_sorted_kernel)
        level_classify<DIM, 0>(L, W, np);
        level_classify<DIM, 1>(L, W, np);
        if constexpr (DIM == 3) level_classify<DIM, 2>(L, W, np);
        HMR_BARRIER();
        const volatile unsigned int* sc = L.sort_count;
        const long n0 = (long)sc[0];
        const long n01 = n0 + (long)sc[1];
        const long nf = n01 + (DIM == 3 ? (long)sc[2] : 0);
        redo_from = min((unsigned long long)sc[3], L.redo.cap);
        level_chunks(L.chunk + CHUNK_SORTED, nf + (long)redo_from, L.chunk_mult, [&](long r) {
            if (r < n0) {
                const long t = (long)L.sorted[L.sort_off[0] + r];
                const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[0]; });
                if (face_item<false, DIM, MODEL, NSP, SCHEME, 0>(P, W[p].g, W[p].S, t - W[p].off_face[0], nullptr))
                    redo_push(L.redo, 0, t);
            } else if (r < n01) {
                const long t = (long)L.sorted[L.sort_off[1] + (r - n0)];
                const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[1]; });
                if (face_item<false, DIM, MODEL, NSP, SCHEME, 1>(P, W[p].g, W[p].S, t - W[p].off_face[1], nullptr))
                    redo_push(L.redo, 1, t);
            } else if (r < nf) {
                if constexpr (DIM == 3) {
                    const long t = (long)L.sorted[L.sort_off[2] + (r - n01)];
                    const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[2]; });
                    if (face_item<false, DIM, MODEL, NSP, SCHEME, 2>(P, W[p].g, W[p].S, t - W[p].off_face[2], nullptr))
                        redo_push(L.redo, 2, t);
                }
            } else {
                level_exact_face<DIM, MODEL, NSP, SCHEME>(P, W, np, L.redo.list[r - nf]);
            }
        });
    } else
#endif
    {
    level_chunks(L.chunk + CHUNK_FACE0, L.total_face[0], L.chunk_mult, [&](long t) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[0]; });
        if (face_item<X, DIM, MODEL, NSP, SCHEME, 0>(P, W[p].g, W[p].S, t - W[p].off_face[0], nullptr))
            redo_push(L.redo, 0, t);
    });
    level_chunks(L.chunk + CHUNK_FACE0 + 1, L.total_face[1], L.chunk_mult, [&](long t) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[1]; });
        if (face_item<X, DIM, MODEL, NSP, SCHEME, 1>(P, W[p].g, W[p].S, t - W[p].off_face[1], nullptr))
            redo_push(L.redo, 1, t);
    });
    if constexpr (DIM == 3) {
        level_chunks(L.chunk + CHUNK_FACE0 + 2, L.total_face[2], L.chunk_mult, [&](long t) {
            const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[2]; });
            if (face_item<X, DIM, MODEL, NSP, SCHEME, 2>(P, W[p].g, W[p].S, t - W[p].off_face[2], nullptr))
                redo_push(L.redo, 2, t);
        });
    }
    }
#if HMR_FAST
    HMR_BARRIER();
    {
        // Exact recomputation of the faces the fast form handed back.
        const unsigned long long nredo = min((unsigned long long)*((volatile unsigned int*)L.redo.count), L.redo.cap);
        const unsigned long long nleft = nredo > redo_from ? nredo - redo_from : 0ull;
        level_chunks(L.chunk + CHUNK_REDO, (long)nleft, L.chunk_mult, [&](long rr) {
            const unsigned long long r = redo_from + (unsigned long long)rr;
            const unsigned long long v = L.redo.list[r];
            const int a = (int)(v >> 56);
            const long t = (long)(v & ((1ull << 56) - 1));
            if (a == 0) {
                const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[0]; });
                face_item<true, DIM, MODEL, NSP, SCHEME, 0>(P, W[p].g, W[p].S, t - W[p].off_face[0], nullptr);
            } else if (a == 1) {
                const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[1]; });
                face_item<true, DIM, MODEL, NSP, SCHEME, 1>(P, W[p].g, W[p].S, t - W[p].off_face[1], nullptr);
            } else if constexpr (DIM == 3) {
                const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_face[2]; });
                face_item<true, DIM, MODEL, NSP, SCHEME, 2>(P, W[p].g, W[p].S, t - W[p].off_face[2], nullptr);
            }
        });
    }
#endif
    HMR_BARRIER();
#undef HMR_BARRIER
    level_cell_items(L.chunk + CHUNK_UPDATE, L.total_update, L, [&](long t) {
        const int p = find_patch(W, np, t, [](const PatchWork& w) { return w.off_update; });
        const PatchWork& w = W[p];
        UpdateArgs U;
        for (int s = 0; s < 3; s++) U.Qint[s] = w.Q[s];
        for (int s = 0; s < 3; s++) U.alpha[s] = L.alpha[s];
        U.nst = L.nst;
        U.beta = L.beta;
        U.dt = L.dt_dev ? *L.dt_dev : L.dt;
        U.Qout = w.Qout;
        U.Fout.p[0] = nullptr;   // flux/source outputs are not produced by the batched form
        U.Sout.p[0] = nullptr;
        U.dorder = DORD;
        update_item<DIM, MODEL, NSP, true>(w.g, w.S, U, t - w.off_update);
    });
}

// The level kernel instantiation of a variant: the diffusive order selects the NavierStokes one.
template <class T, class F>
static int with_dorder(const Variant& v, F f) {
    if constexpr (T::MODEL == SINGLE_SPECIES) {
        if (v.dorder == 4) return f(std::integral_constant<int, 4>{});
        if (v.dorder == 2) return f(std::integral_constant<int, 2>{});
        if (v.dorder == 6) return f(std::integral_constant<int, 6>{});
    }
    if (v.dorder != 0) return -2;
    return f(std::integral_constant<int, 0>{});
}

template <class T, int DORD>
static int level_max_blocks_of(int threads, int* blocks) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, level_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, DORD>, threads, 0);
    if (e != cudaSuccess) return (int)e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    *blocks = per_sm * sms;
    return 0;
}

int level_max_blocks(const Variant& v, int threads, int* blocks) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        return with_dorder<T>(v, [&](auto d) { return level_max_blocks_of<T, decltype(d)::value>(threads, blocks); });
    });
}

int launch_level(const Variant& v, const Params& P, const LevelArgs& L, int blocks, int threads,
                 cudaStream_t st) {
    return dispatch(v, [&](auto t) {
        using T = decltype(t);
        return with_dorder<T>(v, [&](auto d) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(blocks);
            cfg.blockDim = dim3(threads);
            cfg.dynamicSmemBytes = 0;
            cfg.stream = st;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            return (int)cudaLaunchKernelEx(&cfg, level_kernel<T::DIM, T::MODEL, T::NSP, T::SCHEME, decltype(d)::value>,
                                           P, L);
        });
    });
}

}  // namespace HMR_NS
