// staged.cuh -- the neighbour passes with each CTA's candidates staged in
// shared memory by bulk (TMA) copies.
//
// A CTA owns BS consecutive slots [s0, s1) of the cell order. Every candidate
// of its particles lies, for stencil row (dy, dz), in the linear cell range
//   [key(s0) + D - f, key(s1 - 1) + D + f],  D = (dz n1 + dy) n0,
// (a cell (cx + e, cy + dy, cz + dz) has key key + D + e), i.e. one contiguous
// slot range per row. The rows' ranges are merged (they overlap once the CTA
// spans whole rows of cells) and copied to shared memory with one
// cp.async.bulk per range and array, completing on one mbarrier. The passes
// then test candidates and evaluate pairs from shared memory. A CTA whose
// ranges exceed its capacity, or a stencil whose ranges are not in slot order
// (a grid thinner than the stencil), runs the same body on global memory.
// Results do not depend on which of the two a CTA takes.
#pragma once
#include "kernels.cuh"

namespace ag {

constexpr int kStageMaxRows = 49;  // (2f + 1)^(DIM - 1), f <= 3
constexpr unsigned kStageWaitLimit = 1u << 24;  // bounded wait on the copies

struct StageHdr {
    unsigned long long bar;  // mbarrier of the copies
    int total;               // staged slots; -1: this CTA reads global memory
    int ngroups;
    int rlo[kStageMaxRows], rhi[kStageMaxRows];    // slot range of each stencil row
    int glo[kStageMaxRows], gbase[kStageMaxRows];  // merged ranges: first slot, staged index
    int glen[kStageMaxRows];
    int shift[kStageMaxRows];                      // stencil row r: staged = slot + shift[r]
};
constexpr int kStageHdrBytes = (int)((sizeof(StageHdr) + 127) / 128 * 128);

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> this CTA's shared memory (16-byte aligned, size a
// multiple of 16), completing its bytes on the mbarrier.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_test_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase 0 of the mbarrier, at most kStageWaitLimit polls; gives up
// with FLAG_TIMEOUT (the pass's results are then not used by the host).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned* flags) {
    for (unsigned it = 0; it < kStageWaitLimit; ++it) {
        if (mbar_test_wait(bar, 0u)) return true;
        if (it > 64) __nanosleep(64);
    }
    if (flags) atomicOr(flags, (unsigned)FLAG_TIMEOUT);
    return false;
}

// Plans and issues the staging of a CTA's candidates: nsrc arrays of float4
// (srcs[a]), staged array a at body + a * cap float4s. On return (after a
// CTA barrier) H.total >= 0 for the staged path (the copies land on H.bar),
// -1 for the global path.
template <int DIM>
__device__ __forceinline__ void stage_cta(StageHdr& H, float4* body, const float4* const* srcs,
                                          int nsrc, const unsigned* __restrict__ keys,
                                          const int* __restrict__ start, const DevGrid& g,
                                          int s0, int s1, int cap, unsigned* flags) {
    const int tid = threadIdx.x;
    const int f = g.reach, w = 2 * f + 1;
    const int rows = DIM == 2 ? w : w * w;
    if (tid < 32) {
        if (tid == 0) mbar_init(&H.bar, 1);
        const long long K0 = (long long)keys[s0] - g.cell_off;
        const long long K1 = (long long)keys[s1 - 1] - g.cell_off;
        for (int r = tid; r < rows; r += 32) {
            const int dy = r % w - f, dz = (DIM == 3) ? r / w - f : 0;
            const long long D = ((long long)dz * g.n[1] + dy) * g.n[0];
            const long long a = max(K0 + D - f, 0LL), b = min(K1 + D + f, (long long)g.ncells - 1);
            int lo = 0, hi = 0;
            if (g.ok && a <= b) {
                lo = __ldg(start + g.cell_off + a);
                hi = __ldg(start + g.cell_off + b + 1);
            }
            H.rlo[r] = lo;
            H.rhi[r] = hi;
        }
        __syncwarp();
        if (tid == 0) {
            // Merge the row ranges in row order (their slots ascend with the row).
            int total = 0, ng = 0, glo = 0, ghi = 0, last_lo = -1;
            bool ok = true;
            for (int r = 0; r < rows; ++r) {
                const int lo = H.rlo[r], hi = H.rhi[r];
                if (lo >= hi) {
                    H.shift[r] = -1;  // empty row: no candidate reads it
                    continue;
                }
                if (lo < last_lo) {
                    ok = false;
                    break;
                }
                last_lo = lo;
                if (ng > 0 && lo <= ghi) {
                    ghi = max(ghi, hi);
                } else {
                    if (ng > 0) {
                        H.glen[ng - 1] = ghi - glo;
                        total += ghi - glo;
                    }
                    H.glo[ng] = lo;
                    H.gbase[ng] = total;
                    glo = lo;
                    ghi = hi;
                    ++ng;
                }
                H.shift[r] = ng - 1;  // group for now
            }
            if (ng > 0) {
                H.glen[ng - 1] = ghi - glo;
                total += ghi - glo;
            }
            if (!ok || total > cap) {
                H.total = -1;
            } else {
                for (int r = 0; r < rows; ++r)
                    if (H.shift[r] >= 0) H.shift[r] = H.gbase[H.shift[r]] - H.glo[H.shift[r]];
                H.total = total;
                H.ngroups = ng;
                if (total > 0) {
                    mbar_arrive_expect_tx(&H.bar, (unsigned)total * 16u * (unsigned)nsrc);
                    for (int q = 0; q < ng; ++q)
                        for (int a = 0; a < nsrc; ++a)
                            bulk_g2s(body + (size_t)a * cap + H.gbase[q], srcs[a] + H.glo[q],
                                     (unsigned)H.glen[q] * 16u, &H.bar);
                }
            }
        }
    }
    __syncthreads();
}

// Staged float4 arrays of a pass: density xh (+ vm for the 3D mass); force
// xh and vr (2D) or xh, vm, rp (3D).
__host__ __device__ constexpr int stage_arrays(int dim, bool force) {
    return force ? (dim == 2 ? 2 : 3) : (dim == 2 ? 1 : 2);
}
constexpr int kStageSmemBudget = 200 * 1024;  // dynamic shared memory of one CTA at most

// Capacity (staged slots) of a CTA of BS particles: one row's range is about
// the CTA's slots plus 2f cells of halo, the margin covers denser rows;
// bounded by the shared-memory budget.
__host__ __device__ constexpr int stage_cap(int dim, int reach, int bs, bool force) {
    const int rows = dim == 2 ? 2 * reach + 1 : (2 * reach + 1) * (2 * reach + 1);
    const int want = rows * (bs + bs / 4 + 32);
    const int lists = (force ? kListCap : 2 * kListCapD) * bs * 2;
    const int fit = (kStageSmemBudget - kStageHdrBytes - lists) / (16 * stage_arrays(dim, force));
    return want < fit ? want : fit;
}

// Dynamic shared memory of a staged pass: the staged arrays and the lists
// (16-bit staged indices), or the int lists of the global path, whichever
// is larger.
__host__ __device__ constexpr int stage_smem_bytes(int dim, int reach, int bs, bool force) {
    const int staged = stage_cap(dim, reach, bs, force) * 16 * stage_arrays(dim, force) +
                       (force ? kListCap : 2 * kListCapD) * bs * 2;
    const int global = (force ? kListCap : 2 * kListCapD) * bs * 4;
    return kStageHdrBytes + (staged > global ? staged : global);
}

template <int DIM, int BS>
__global__ void __launch_bounds__(BS, 1024 / BS)
    k_density_st(StateB B, const unsigned* __restrict__ keys, const int* __restrict__ start,
                 const DevGrid* __restrict__ gp, DevParams P, int n, int cap,
                 unsigned* __restrict__ flags) {
    extern __shared__ __align__(128) unsigned char smem[];
    StageHdr& H = *reinterpret_cast<StageHdr*>(smem);
    float4* body = reinterpret_cast<float4*>(smem + kStageHdrBytes);
    const int s0 = blockIdx.x * BS, s1 = min(s0 + BS, n);
    const DevGrid g = load_grid<false>(gp);
    constexpr int NS = stage_arrays(DIM, false);
    const float4* srcs[2] = {B.xh, B.vm};
    stage_cta<DIM>(H, body, srcs, NS, keys, start, g, s0, s1, cap, flags);
    const int s = s0 + (int)threadIdx.x;
    const int total = H.total;
    if (total > 0 && !mbar_wait_bounded(&H.bar, flags)) return;  // host reports the timeout
    if (total >= 0) {
        const StageView SV{body, NS > 1 ? body + cap : nullptr, nullptr, H.shift};
        auto* lists = reinterpret_cast<unsigned short (*)[BS]>(body + (size_t)NS * cap);
        density_body<DIM, 1, BS, true, false, true, unsigned short>(
            B, keys, start, g, P, s, s < n, lists, lists + kListCapD, SV);
    } else {
        auto* lists = reinterpret_cast<int (*)[BS]>(body);
        density_body<DIM, 1, BS, true, false>(B, keys, start, g, P, s, s < n, lists,
                                              lists + kListCapD);
    }
}

template <int DIM, int BS>
__global__ void __launch_bounds__(BS, 1024 / BS)
    k_force_st(StateB B, StateA A, const unsigned* __restrict__ keys, const int* __restrict__ start,
               const DevGrid* __restrict__ gp, DevParams P, StepArgs S, unsigned* __restrict__ flags,
               int n, int cap) {
    extern __shared__ __align__(128) unsigned char smem[];
    StageHdr& H = *reinterpret_cast<StageHdr*>(smem);
    float4* body = reinterpret_cast<float4*>(smem + kStageHdrBytes);
    const int s0 = blockIdx.x * BS, s1 = min(s0 + BS, n);
    const DevGrid g = load_grid<false>(gp);
    constexpr int NS = stage_arrays(DIM, true);
    const float4* srcs[3] = {B.xh, DIM == 2 ? B.vr : B.vm, B.rp};
    stage_cta<DIM>(H, body, srcs, NS, keys, start, g, s0, s1, cap, flags);
    const int s = s0 + (int)threadIdx.x;
    const int total = H.total;
    if (total > 0 && !mbar_wait_bounded(&H.bar, flags)) return;  // host reports the timeout
    if (total >= 0) {
        const StageView SV{body, body + cap, NS > 2 ? body + 2 * (size_t)cap : nullptr, H.shift};
        auto* lists = reinterpret_cast<unsigned short (*)[BS]>(body + (size_t)NS * cap);
        force_body<DIM, 1, BS, true, false, true, unsigned short>(B, A, keys, start, g, P, S,
                                                                   flags, s, s < n, lists, SV);
    } else {
        auto* lists = reinterpret_cast<int (*)[BS]>(body);
        force_body<DIM, 1, BS, true, false>(B, A, keys, start, g, P, S, flags, s, s < n, lists);
    }
}

}  // namespace ag
