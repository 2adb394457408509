// Register-resident split sweeps of the 9-point evaluator (KIND 4): d8 (with
// the exact fixed-point RHS on the FP32 path), the compact and the Gaussian
// filters.  The kernel is in pg_split.cuh.
#include "pg_split.cuh"

namespace pg {
namespace {
template <int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, bool EXACT>
int launch_seg(const SParams& P, const SplitSet& ss, void* stream) {
  const size_t smem = DIR == 0 ? ss.smem_seg_x : ss.smem_seg_yz;
  auto k = seg_kernel<KIND, PER, IMPL, ADDBACK, DIR, EPI, EXACT>;
  static size_t attr = 0;
  if (smem > attr) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error("split sweep: %s (%zu bytes of shared memory)", cudaGetErrorString(e), smem);
      return PG_ECUDA;
    }
    attr = smem;
  }
  k<<<ss.ntiles, kSplitThreads, smem, (cudaStream_t)stream>>>(P);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("split sweep launch: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

template <int KIND, bool PER, bool IMPL, bool ADDBACK, unsigned EPIS, bool EXACT = false, int DIR>
int seg_epi(const SParams& P, const SplitSet& ss, int epi, void* st) {
  if constexpr ((EPIS >> EPI_STORE) & 1u)
    if (epi == EPI_STORE) return launch_seg<KIND, PER, IMPL, ADDBACK, DIR, EPI_STORE, EXACT>(P, ss, st);
  if constexpr ((EPIS >> EPI_ADD) & 1u)
    if (epi == EPI_ADD) return launch_seg<KIND, PER, IMPL, ADDBACK, DIR, EPI_ADD, EXACT>(P, ss, st);
  if constexpr ((EPIS >> EPI_RING_SET) & 1u)
    if (epi == EPI_RING_SET) return launch_seg<KIND, PER, IMPL, ADDBACK, DIR, EPI_RING_SET, EXACT>(P, ss, st);
  if constexpr ((EPIS >> EPI_RING_MAX) & 1u)
    if (epi == EPI_RING_MAX) return launch_seg<KIND, PER, IMPL, ADDBACK, DIR, EPI_RING_MAX, EXACT>(P, ss, st);
  set_error("split sweep: epilogue %d is not built for this operator", epi);
  return PG_EINVAL;
}

template <int KIND, bool PER, bool IMPL, bool ADDBACK, unsigned EPIS, bool EXACT = false>
int seg_dir_epi(const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
  if (dir == 0) return seg_epi<KIND, PER, IMPL, ADDBACK, EPIS, EXACT, 0>(P, ss, epi, st);
  if (dir == 1) return seg_epi<KIND, PER, IMPL, ADDBACK, EPIS, EXACT, 1>(P, ss, epi, st);
  return seg_epi<KIND, PER, IMPL, ADDBACK, EPIS, EXACT, 2>(P, ss, epi, st);
}
}  // namespace

int seg_launch_r4(const OpRef& op, const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
  switch (op.kind) {
    case OPK_D8:
      if (op.exact)
        return op.periodic ? seg_dir_epi<4, true, true, false, kEpiRing, true>(P, ss, dir, epi, st)
                           : seg_dir_epi<4, false, true, false, kEpiRing, true>(P, ss, dir, epi, st);
      return op.periodic ? seg_dir_epi<4, true, true, false, kEpiRing>(P, ss, dir, epi, st)
                         : seg_dir_epi<4, false, true, false, kEpiRing>(P, ss, dir, epi, st);
    case OPK_SF:
      return op.periodic ? seg_dir_epi<4, true, true, true, kEpiStore>(P, ss, dir, epi, st)
                         : seg_dir_epi<4, false, true, true, kEpiStore>(P, ss, dir, epi, st);
    case OPK_GF:
      return op.periodic ? seg_dir_epi<4, true, false, true, kEpiStore>(P, ss, dir, epi, st)
                         : seg_dir_epi<4, false, false, true, kEpiStore>(P, ss, dir, epi, st);
    default:
      set_error("split sweep: operator %d is not a 9-point operator", op.kind);
      return PG_EINVAL;
  }
}

}  // namespace pg
