// sed_observables.cu -- the device side of the flux-torus observables.
//
// * position_operator: _position_operator_matrix (observables/charge_pump.jl:
//   47-91), Resta's periodic position operator U_d = exp(2 pi i X_d / L_d)
//   projected between two symmetry sectors of one catalog.  U_d is diagonal
//   in the Fock basis, so it maps every orbit to itself: the projected matrix
//   has at most one entry per column, at the row of the same representative
//   in the target sector, with the value
//     (1/|G|) sum_g chi_to(g) conj(chi_from(g)) prod_{j in g(rep)} phase_j.
//   One thread per column evaluates the |G| images and their site-phase
//   products, in the reference's order (products lsb first, separately
//   rounded complex products, the 1e-13 sparsity cut).
// * fock_overlaps: _subspace_overlap_matrix and _fock_amplitude_overlap
//   (observables/many_body_chern_number.jl:46-71), the overlap matrix
//   M_ij = <a_i|b_j> of two sets of states given as dense Fock-amplitude
//   vectors (colex-rank order, the form sector_expand_fock writes).  A
//   reference Dict holds only the nonzero amplitudes; the dense sum adds
//   exact zeros for the others.  Partial sums per block in fixed order, then
//   one fixed-order reduction, so results do not depend on the launch.
#include <cmath>
#include <vector>

#include "sed_internal.cuh"

namespace sed {

namespace {

constexpr int kObsBS = 256;

__global__ void __launch_bounds__(kObsBS) k_position_operator(int64_t dim_from, int N, int G,
                                                              const uint32_t* __restrict__ row_orbit_from,
                                                              const int32_t* __restrict__ orbit_row_to,
                                                              const uint64_t* __restrict__ reps,
                                                              const uint8_t* __restrict__ perm_g,
                                                              const double2* __restrict__ site_phase,
                                                              const double2* __restrict__ chi_to,
                                                              const double2* __restrict__ chi_from, double inv_nG,
                                                              int64_t* __restrict__ row_out,
                                                              double2* __restrict__ elem_out) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  __shared__ double2 sph[64];
  __shared__ double2 sw[SED_MAX_OPS];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  for (int i = threadIdx.x; i < N; i += blockDim.x) sph[i] = site_phase[i];
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double2 a = chi_to[g], b = chi_from[g];
    sw[g] = dev::cmul_rn(a, make_double2(b.x, -b.y));  // chi_to(g) * conj(chi_from(g))
  }
  __syncthreads();
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim_from;
       r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t o = row_orbit_from[r];
    const int32_t to = orbit_row_to[o];
    if (to < 0) {
      row_out[r] = -1;
      elem_out[r] = make_double2(0.0, 0.0);
      continue;
    }
    const uint64_t m = reps[o];
    double2 elem = make_double2(0.0, 0.0);
    for (int g = 0; g < G; ++g) {
      uint64_t sh = dev::apply_perm(m, sperm + g * 64);
      double2 z = make_double2(1.0, 0.0);
      while (sh) {  // _position_phase_for_mask: lsb first
        const int i = __ffsll((long long)sh) - 1;
        sh &= sh - 1;
        z = dev::cmul_rn(z, sph[i]);
      }
      const double2 t = dev::cmul_rn(sw[g], z);
      elem = make_double2(__dadd_rn(elem.x, t.x), __dadd_rn(elem.y, t.y));
    }
    elem = make_double2(__dmul_rn(elem.x, inv_nG), __dmul_rn(elem.y, inv_nG));
    if (hypot(elem.x, elem.y) > 1e-13) {
      row_out[r] = to;
      elem_out[r] = elem;
    } else {
      row_out[r] = -1;
      elem_out[r] = make_double2(0.0, 0.0);
    }
  }
}

__global__ void k_orbit_row_fill(int64_t n_orb, int32_t* __restrict__ orbit_row) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_orb; o += (int64_t)gridDim.x * blockDim.x)
    orbit_row[o] = -1;
}
__global__ void k_orbit_row_set(int64_t dim, const uint32_t* __restrict__ row_orbit, int32_t* __restrict__ orbit_row) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
    orbit_row[row_orbit[r]] = (int32_t)r;
}

// partial sums of conj(a_i) b_j over a block's slice of the Fock states, one
// block row per (i, j) pair
__global__ void __launch_bounds__(kObsBS) k_fock_overlap_part(int64_t n, const double2* __restrict__ A, int nb,
                                                              const double2* __restrict__ B,
                                                              double2* __restrict__ part) {
  const int pair = blockIdx.y, i = pair / nb, j = pair % nb;
  const double2* a = A + (size_t)i * n;
  const double2* b = B + (size_t)j * n;
  double re = 0.0, im = 0.0;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = a[s], y = b[s];
    // conj(x) y
    re += x.x * y.x + x.y * y.y;
    im += x.x * y.y - x.y * y.x;
  }
  __shared__ double sr[kObsBS / 32], si[kObsBS / 32];
  for (int off = 16; off > 0; off >>= 1) {
    re += __shfl_xor_sync(0xFFFFFFFFu, re, off);
    im += __shfl_xor_sync(0xFFFFFFFFu, im, off);
  }
  if ((threadIdx.x & 31) == 0) {
    sr[threadIdx.x >> 5] = re;
    si[threadIdx.x >> 5] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < kObsBS / 32; ++w) {
      tr += sr[w];
      ti += si[w];
    }
    part[(size_t)pair * gridDim.x + blockIdx.x] = make_double2(tr, ti);
  }
}

__global__ void k_fock_overlap_reduce(int nblk, const double2* __restrict__ part, double2* __restrict__ out) {
  const int pair = blockIdx.x;
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int b = 0; b < nblk; ++b) {
      const double2 v = part[(size_t)pair * nblk + b];
      tr += v.x;
      ti += v.y;
    }
    out[pair] = make_double2(tr, ti);
  }
}

}  // namespace

void position_operator(const SectorImpl& to, const SectorImpl& from, const double* site_phase, int64_t* row_out,
                       double* elem_out) {
  const CatalogImpl& C = *from.cat;
  const GroupImpl& G = *from.group;
  SED_REQUIRE(to.cat.get() == from.cat.get(), 1, "both sectors must come from the same orbit catalog");
  SED_REQUIRE(to.group->n_ops == G.n_ops && to.group->n_site == G.n_site && to.group->perm == G.perm, 1,
              "both sectors must use the same symmetry group");
  SED_REQUIRE(site_phase && row_out && elem_out, 1, "NULL argument");
  const int64_t dim = from.dim;
  if (dim == 0) return;
  cudaStream_t s = C.stream;
  DevBuf orow((size_t)std::max<int64_t>(C.n_orbits, 1) * 4), dph, dchi_to, dchi_from,
      drow((size_t)dim * 8), delem((size_t)dim * 16);
  k_orbit_row_fill<<<grid1(C.n_orbits, 256), 256, 0, s>>>(C.n_orbits, orow.as<int32_t>());
  if (to.dim > 0)
    k_orbit_row_set<<<grid1(to.dim, 256), 256, 0, s>>>(to.dim, to.row_orbit.as<uint32_t>(), orow.as<int32_t>());
  SED_CUDA(cudaGetLastError());
  std::vector<double> ph(site_phase, site_phase + 2 * (size_t)G.n_site);
  upload(dph, ph, s);
  upload(dchi_to, to.chi, s);
  upload(dchi_from, from.chi, s);
  k_position_operator<<<grid1(dim, kObsBS), kObsBS, 0, s>>>(
      dim, G.n_site, G.n_ops, from.row_orbit.as<uint32_t>(), orow.as<int32_t>(), C.reps.as<uint64_t>(),
      C.perm_u8.as<uint8_t>(), dph.as<double2>(), dchi_to.as<double2>(), dchi_from.as<double2>(),
      1.0 / (double)G.n_ops, drow.as<int64_t>(), delem.as<double2>());
  SED_CUDA(cudaGetLastError());
  SED_CUDA(cudaMemcpyAsync(row_out, drow.p, (size_t)dim * 8, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaMemcpyAsync(elem_out, delem.p, (size_t)dim * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

void fock_overlaps(const double* A, int na, const double* B, int nb, int64_t n, int is_device, double* M) {
  SED_REQUIRE(na >= 0 && nb >= 0 && n >= 0, 1, "negative size");
  SED_REQUIRE(na * nb <= 65535, 5, "at most 65535 overlaps per call");
  SED_REQUIRE((na == 0 || A) && (nb == 0 || B) && M, 1, "NULL argument");
  if (na == 0 || nb == 0) return;
  if (n == 0) {
    for (int i = 0; i < 2 * na * nb; ++i) M[i] = 0.0;
    return;
  }
  cudaStream_t s = cudaStreamPerThread;
  DevBuf da, db;
  const double2* pa = reinterpret_cast<const double2*>(A);
  const double2* pb = reinterpret_cast<const double2*>(B);
  if (!is_device) {
    da.alloc((size_t)na * n * 16);
    db.alloc((size_t)nb * n * 16);
    SED_CUDA(cudaMemcpyAsync(da.p, A, (size_t)na * n * 16, cudaMemcpyHostToDevice, s));
    SED_CUDA(cudaMemcpyAsync(db.p, B, (size_t)nb * n * 16, cudaMemcpyHostToDevice, s));
    pa = da.as<double2>();
    pb = db.as<double2>();
  }
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((n + kObsBS - 1) / kObsBS, device_sm_count() * 2));
  DevBuf part((size_t)nblk * na * nb * 16), out((size_t)na * nb * 16);
  k_fock_overlap_part<<<dim3(nblk, na * nb), kObsBS, 0, s>>>(n, pa, nb, pb, part.as<double2>());
  k_fock_overlap_reduce<<<na * nb, 32, 0, s>>>(nblk, part.as<double2>(), out.as<double2>());
  SED_CUDA(cudaGetLastError());
  SED_CUDA(cudaMemcpyAsync(M, out.p, (size_t)na * nb * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

}  // namespace sed
