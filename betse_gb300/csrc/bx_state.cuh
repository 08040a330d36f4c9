// bx_state.cuh -- BETSE's state arrays to and from the device layouts, on the
// device (bx_state_upload / bx_state_download).
//
// The caller's arrays cross the bus as they are (vm [M], cc_cells [I][C],
// cc_at_mem [I][M], gjopen [M]); these kernels check them and re-lay them:
// cc_at_mem is one value per cell in BETSE (update_intra, sim.py:2310), so
// the cell's first membrane gives it; the split form also keeps one Vmem per
// cell (sim.py:2027-2029) in the 32-byte cell records and each concentration
// as an FP32 (hi, lo) pair.  The conversions are those of a host cast (round
// to nearest), so the device state is the same bit for bit.
#pragma once
#include <cstdint>

namespace bx {

struct StateIO {
  int C, M, I, S, rec;              // cells, membranes, ions, cell slots, floats per record
  const int* cell_ptr;              // [C+1]
  const int* m2c;                   // [M]
  const int* map_env;               // [M]
  const double* phib;               // [G] boundary potential (read when phib_on)
  int phib_on;
  const int* slot_of_cell;          // [C] split form
  const int* slot_of_mem;           // [M] split form
};

__device__ __forceinline__ double state_phib(const StateIO& io, int m) {
  return io.phib_on ? io.phib[io.map_env[m]] : 0.0;
}

// The checks of bx_state_upload, one thread per membrane: flag[0] when
// cc_at_mem differs from its cell's first membrane (a NaN differs too), flag[1]
// (with check_vm, the split form) when vm + Phi_b is not uniform over the cell.
__global__ void k_state_check(StateIO io, const double* __restrict__ vm, const double* __restrict__ cam,
                              int check_vm, int* flag) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= io.M) return;
  const int f = io.cell_ptr[io.m2c[m]];
  if (m == f) return;
  for (int i = 0; i < io.I; ++i)
    if (cam[(size_t)i * io.M + m] != cam[(size_t)i * io.M + f]) { atomicOr(&flag[0], 1); break; }
  if (check_vm) {
    const double v0 = vm[f] + state_phib(io, f), v = vm[m] + state_phib(io, m);
    if (fabs(v - v0) > 1e-12 * fabs(v0) + 1e-18) atomicOr(&flag[1], 1);
  }
}

// plain form: the membrane-side concentration of each cell
__global__ void k_state_pack_ccm(StateIO io, const double* __restrict__ cam, double* ccm) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= io.C) return;
  const int f = io.cell_ptr[c];
  for (int i = 0; i < io.I; ++i) ccm[(size_t)i * io.C + c] = cam[(size_t)i * io.M + f];
}

// split form, one thread per cell: record (membrane-side concentrations, Vmem)
// and the (hi, lo) concentration pairs; padding slots are zeroed beforehand
__global__ void k_state_pack_split(StateIO io, const double* __restrict__ vm, const double* __restrict__ cc,
                                   const double* __restrict__ cam, float* rec, float2* cc2) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= io.C) return;
  const int f = io.cell_ptr[c];
  const int sc = io.slot_of_cell[c];
  rec[(size_t)sc * io.rec + io.rec - 1] = (float)(vm[f] + state_phib(io, f));
  for (int i = 0; i < io.I; ++i) {
    rec[(size_t)sc * io.rec + i] = (float)cam[(size_t)i * io.M + f];
    const double x = cc[(size_t)i * io.C + c];
    const float hi = (float)x;
    cc2[(size_t)i * io.S + sc] = make_float2(hi, (float)(x - (double)hi));
  }
}

// split form, gap-junction open fraction per membrane slot (gjopen, or the
// static weights when the caller gives none)
__global__ void k_state_pack_gjo(StateIO io, const double* __restrict__ go, float* slot_go) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= io.M) return;
  slot_go[io.slot_of_mem[m]] = (float)go[m];
}

// plain form: cc_at_mem broadcast from the cell values
__global__ void k_state_unpack_cam(StateIO io, const double* __restrict__ ccm, double* cam) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= io.M) return;
  const int c = io.m2c[m];
  for (int i = 0; i < io.I; ++i) cam[(size_t)i * io.M + m] = ccm[(size_t)i * io.C + c];
}

// split form: threads below M write the membrane arrays (vm, cc_at_mem, and
// gjopen when slot_go is given), threads below C the cell concentrations
__global__ void k_state_unpack_split(StateIO io, const float* __restrict__ rec, const float2* __restrict__ cc2,
                                     const float* __restrict__ slot_go, double* vm, double* cam, double* cc,
                                     double* go) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < io.M) {
    const int sc = io.slot_of_cell[io.m2c[t]];
    const float* r = rec + (size_t)sc * io.rec;
    vm[t] = (double)r[io.rec - 1] - state_phib(io, t);
    for (int i = 0; i < io.I; ++i) cam[(size_t)i * io.M + t] = (double)r[i];
    if (slot_go) go[t] = (double)slot_go[io.slot_of_mem[t]];
  }
  if (t < io.C) {
    const int sc = io.slot_of_cell[t];
    for (int i = 0; i < io.I; ++i) {
      const float2 x = cc2[(size_t)i * io.S + sc];
      cc[(size_t)i * io.C + t] = (double)x.x + (double)x.y;
    }
  }
}

}  // namespace bx
