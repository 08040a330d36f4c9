// bx_launch.cuh -- host-side launcher of the templated plain-form step kernel;
// the instantiations live in bx_step_f64.cu so they compile in parallel with
// the rest of the library.
#pragma once
#include "bx_kernels.cuh"

namespace bx {

// per-ion flux rows, the cell Vmem row, and scratch rows: four for outputs,
// seven for outputs with polarizability (at most 48 KB: 8 ions, 256 threads)
inline size_t cell_step_smem(int I, int tpb, bool out, bool polar) {
  const size_t scratch = polar ? (out ? 7 : 4) : (out ? 4 : 0);
  return sizeof(double) * (size_t)tpb * (2 * (size_t)I + 1 + scratch);
}

template <typename T, int TPB>
cudaError_t launch_cell_step(bool ecm, bool out, bool phib, int nblk, cudaStream_t s,
                             const DevGeom& g, const StepPtrs& p, const StepConst& k);

#define BX_DEFINE_CELL_STEP_LAUNCHER(T, TPB)                                                    \
  template <>                                                                                   \
  cudaError_t launch_cell_step<T, TPB>(bool ecm, bool out, bool phib, int nblk, cudaStream_t s, \
                                       const DevGeom& g, const StepPtrs& p, const StepConst& k) { \
    const size_t sm = cell_step_smem(k.I, TPB, out, k.polar != 0);                                            \
    const int code = (ecm ? 4 : 0) | (out ? 2 : 0) | (phib ? 1 : 0);                            \
    switch (code) {                                                                             \
      case 0: k_cell_step<T, TPB, false, false, false><<<nblk, TPB, sm, s>>>(g, p, k); break;  \
      case 1: k_cell_step<T, TPB, false, false, true><<<nblk, TPB, sm, s>>>(g, p, k); break;   \
      case 2: k_cell_step<T, TPB, false, true, false><<<nblk, TPB, sm, s>>>(g, p, k); break;   \
      case 3: k_cell_step<T, TPB, false, true, true><<<nblk, TPB, sm, s>>>(g, p, k); break;    \
      case 4: k_cell_step<T, TPB, true, false, false><<<nblk, TPB, sm, s>>>(g, p, k); break;   \
      case 5: k_cell_step<T, TPB, true, false, true><<<nblk, TPB, sm, s>>>(g, p, k); break;    \
      case 6: k_cell_step<T, TPB, true, true, false><<<nblk, TPB, sm, s>>>(g, p, k); break;    \
      default: k_cell_step<T, TPB, true, true, true><<<nblk, TPB, sm, s>>>(g, p, k); break;    \
    }                                                                                           \
    return cudaGetLastError();                                                                  \
  }

// the plain step for small clusters (k_cell_step_ion), MB membrane slots; it
// also mixes the well-mixed environment
template <int MB>
cudaError_t launch_cell_step_ion(int nblk, cudaStream_t s, const DevGeom& g, const StepPtrs& p, const StepConst& k,
                                 const EnvMix& em);

#define BX_DEFINE_CELL_STEP_ION_LAUNCHER(MB)                                                       \
  template <>                                                                                      \
  cudaError_t launch_cell_step_ion<MB>(int nblk, cudaStream_t s, const DevGeom& g, const StepPtrs& p, \
                                       const StepConst& k, const EnvMix& em) {                     \
    k_cell_step_ion<MB><<<nblk, MB * 8, 0, s>>>(g, p, k, em);                                      \
    return cudaGetLastError();                                                                     \
  }

}  // namespace bx
