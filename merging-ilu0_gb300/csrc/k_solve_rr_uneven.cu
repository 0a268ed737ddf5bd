// Uneven-batch kernel of the register-resident solver (k_solve_rr.cuh), in a
// translation unit of its own so that it compiles in parallel with the rest.
#include "k_solve_rr.cuh"

namespace bilu {
namespace {

// Systems of an uneven-batch bucket (own size and pattern each), merged
// ILU(0) (PV 3) or none (PV 0), no optional staging.  A grid of one CTA per
// system solves system order[b] on CTA b (longest first); a smaller,
// persistent grid takes the bucket's systems from its atomic work queue
// (u.counter, zeroed before the launch), one at a time per CTA.  The queue
// slot is an unused broadcast word of the reduction area (rr_red_bytes: 16
// scalars after the partial sums, of which rr_solve uses 8).
template <int R, int PV, typename FT>
__global__ void BILU_RR_BOUNDS k_bicgstab_rr_uneven(const UnevenArgs u) {
  extern __shared__ __align__(16) unsigned char smem[];
  volatile int* slot = reinterpret_cast<volatile int*>(reinterpret_cast<double*>(smem) + 2 * blockDim.x + 15);
  const bool queue = (int)gridDim.x < u.count;
  int b = blockIdx.x;
  if (queue) {
    if (threadIdx.x == 0) *slot = atomicAdd(u.counter, 1);
    __syncthreads();
    b = *slot;
  }
  while (b < u.count) {
    const int sys = __ldg(u.order + b);
    const SysDesc d = u.desc[sys];
    DevPattern P;
    P.n = d.n;
    P.nnz = P.a_nnz = d.nnz;
    P.a_maxl = d.maxl;
    P.rp = P.a_rp = u.meta + d.o_rp;
    P.ci = P.a_ci = u.meta + d.o_ci;
    P.diag = u.meta + d.o_diag;
    P.nlev_lo = d.nlev_lo;
    P.nlev_up = d.nlev_up;
    P.maxw_lo = P.maxw_up = d.maxw;
    P.lev_lo_ptr = u.meta + d.o_llp;
    P.lev_lo_rows = u.meta + d.o_llr;
    P.lev_up_ptr = u.meta + d.o_lup;
    P.lev_up_rows = u.meta + d.o_lur;
    P.dep_ptr = u.meta + d.o_dp;
    P.dep = reinterpret_cast<const int2*>(u.meta + d.o_dep);
    P.tp_lo_hdr = reinterpret_cast<const int2*>(u.meta + d.o_tlh);
    P.tp_lo = u.meta + d.o_tl;
    P.tp_up_hdr = reinterpret_cast<const int2*>(u.meta + d.o_tuh);
    P.tp_up = u.meta + d.o_tu;
    if (d.o_ip >= 0) {
      P.ilu_hdr = reinterpret_cast<const int4*>(u.meta + d.o_ih);
      P.ilu_prog = u.meta + d.o_ip;
      P.ilu_prog_approach = u.base.approach;
    }
    const RRLayout L = rr_layout_base(d.n, d.nnz, PV, sizeof(FT) == 4, true, blockDim.x);
    rr_solve<R, PV, FT, false, false>(u.base, P, L, smem, sys, u.base.A + d.val_off, u.base.b + d.vec_off,
                                      u.base.x + d.vec_off);
    if (!queue) break;
    __syncthreads();  // every thread is done with this system (shared memory, the slot)
    if (threadIdx.x == 0) *slot = atomicAdd(u.counter, 1);
    __syncthreads();
    b = *slot;
  }
}

template <int PV, typename FT>
const void* rr_uneven_kernel_pv(int R) {
  switch (R) {
    case 1: return (const void*)k_bicgstab_rr_uneven<1, PV, FT>;
    case 2: return (const void*)k_bicgstab_rr_uneven<2, PV, FT>;
    case 4: return (const void*)k_bicgstab_rr_uneven<4, PV, FT>;
    default: return (const void*)k_bicgstab_rr_uneven<8, PV, FT>;
  }
}

}  // namespace

const void* rr_uneven_kernel(int pv, int fp32, int R) {
  if (pv == 0) return rr_uneven_kernel_pv<0, double>(R);
  return fp32 ? rr_uneven_kernel_pv<3, float>(R) : rr_uneven_kernel_pv<3, double>(R);
}

// Dynamic shared memory = u.smem_budget (the bucket's largest layout); the
// caller has set the kernel's shared-memory attribute outside any capture.
// grid: u.count (one CTA per system) or fewer persistent CTAs over the queue.
cudaError_t launch_uneven_rr(const UnevenArgs& u, int nt, int R, int pv, int fp32, int grid, cudaStream_t st) {
  if (u.count == 0) return cudaSuccess;
  if (grid <= 0 || grid > u.count) grid = u.count;
  void* args[] = {const_cast<UnevenArgs*>(&u)};
  return cudaLaunchKernel(rr_uneven_kernel(pv, fp32, R), dim3(grid), dim3(nt), args, (size_t)u.smem_budget, st);
}

}  // namespace bilu
