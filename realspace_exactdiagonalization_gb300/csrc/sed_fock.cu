// sed_fock.cu -- a sector vector expanded to Fock amplitudes.
//
// _expand_sector_state_to_fock_amplitudes (observables/entanglement_spectrum.jl:46-79)
// spreads every sector coefficient over the group images of its orbit
// representative, c / sqrt(|G| stab) * conj(chi(g)) * alpha_g(rep) for each g,
// sums the copies that land on one mask, drops |amp| <= atol and normalises.
// Here that scatter becomes a gather over the fixed-filling states: the state
// word of rank s names its orbit and one group element g0 with g0(rep) = s;
// the stab(rep) elements of the coset g0 Stab(rep) all contribute the same
// amplitude (the sector's compatibility condition chi(h) = alpha_h(rep) on the
// stabilizer), so amp(s) = stab * c / sqrt(|G| stab) * conj(chi(g0)) *
// alpha_g0(rep).  One thread per state: one 8-byte state word, one gathered
// coefficient and one 16-byte write, HBM-bound.  The output is the dense
// vector over colex ranks (rank r = the r-th k-subset in ascending mask order),
// the GPU counterpart of the reference's Dict{Mask, ComplexF64}.
#include <cmath>
#include <vector>

#include "sed_internal.cuh"

namespace sed {

void expand_vec(const SectorImpl& S, const double* xsec, double* xpad, cudaStream_t s);

namespace {

constexpr int kFockBS = 256;

__global__ void __launch_bounds__(kFockBS) k_fock_expand(int64_t n_states, int N, int G, int fermi,
                                                         const uint64_t* __restrict__ state,
                                                         const uint64_t* __restrict__ reps,
                                                         const uint8_t* __restrict__ stab,
                                                         const uint8_t* __restrict__ rowflag,
                                                         const uint8_t* __restrict__ perm_g,
                                                         const double2* __restrict__ phase,
                                                         const double2* __restrict__ chi,
                                                         const double2* __restrict__ xpad, double atol,
                                                         double2* __restrict__ out, double* __restrict__ part) {
  __shared__ uint8_t sperm[SED_MAX_OPS * 64];
  __shared__ double2 schi[SED_MAX_OPS];
  __shared__ double red[kFockBS / 32];
  for (int i = threadIdx.x; i < G * 64; i += blockDim.x) sperm[i] = perm_g[i];
  for (int i = threadIdx.x; i < G; i += blockDim.x) schi[i] = chi[i];
  __syncthreads();
  double n2 = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_states;
       r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t w = state[r];
    const uint32_t o = (uint32_t)w;
    double2 amp = make_double2(0.0, 0.0);
    if (rowflag[o]) {
      const double2 c = xpad[o];
      if (hypot(c.x, c.y) > atol) {
        const int g = (int)((w >> 32) & 0xFF);
        const int so = stab[o];
        double2 al;
        dev::apply_full(reps[o], sperm + g * 64, phase + (size_t)g * N, fermi, &al);
        const double d = sqrt((double)(G * so));
        const double2 pre = make_double2(c.x / d, c.y / d);
        const double2 ch = schi[g];
        // (pre * conj(chi(g))) * alpha, as the reference evaluates it
        const double2 t = make_double2(__dadd_rn(__dmul_rn(pre.x, ch.x), __dmul_rn(pre.y, ch.y)),
                                       __dsub_rn(__dmul_rn(pre.y, ch.x), __dmul_rn(pre.x, ch.y)));
        const double2 a = dev::cmul_rn(t, al);
        amp = make_double2(a.x * so, a.y * so);
        if (!(hypot(amp.x, amp.y) > atol)) amp = make_double2(0.0, 0.0);
      }
    }
    out[r] = amp;
    n2 += amp.x * amp.x + amp.y * amp.y;
  }
  // fixed-order block partial (warp shuffle tree, then warp order)
  for (int off = 16; off > 0; off >>= 1) n2 += __shfl_xor_sync(0xFFFFFFFFu, n2, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = n2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < kFockBS / 32; ++i) s += red[i];
    part[blockIdx.x] = s;
  }
}

__global__ void k_fock_scale(int64_t n, double2* __restrict__ out, double inv) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = out[r];
    out[r] = make_double2(v.x * inv, v.y * inv);
  }
}

}  // namespace

void sector_expand_fock(const SectorImpl& S, const double* c, int64_t dim, double atol, double* out,
                        int64_t n_states, int is_device, double* norm2_out) {
  const CatalogImpl& C = *S.cat;
  const GroupImpl& G = *S.group;
  SED_REQUIRE(dim == S.dim, 1, "coefficient vector length differs from the sector dimension");
  SED_REQUIRE(n_states == C.n_states, 1, "output length differs from the number of fixed-filling states");
  SED_REQUIRE(dim == 0 || c, 1, "NULL coefficient vector");
  SED_REQUIRE(out, 1, "NULL output");
  SED_REQUIRE(atol >= 0.0, 1, "atol must be non-negative");
  cudaStream_t s = S.stream();
  const int64_t n_orb = C.n_orbits;
  DevBuf xpad((size_t)std::max<int64_t>(n_orb, 1) * 16), csec, outd;
  const double* cdev = c;
  if (!is_device && dim) {
    csec.alloc((size_t)dim * 16);
    SED_CUDA(cudaMemcpyAsync(csec.p, c, (size_t)dim * 16, cudaMemcpyHostToDevice, s));
    cdev = csec.as<double>();
  }
  expand_vec(S, cdev, xpad.as<double>(), s);
  double2* o = reinterpret_cast<double2*>(out);
  if (!is_device) {
    outd.alloc((size_t)std::max<int64_t>(n_states, 1) * 16);
    o = outd.as<double2>();
  }
  std::vector<double> chi = S.chi;
  DevBuf dchi;
  upload(dchi, chi, s);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n_states + kFockBS - 1) / kFockBS,
                                                                (int64_t)device_sm_count() * 16));
  DevBuf part((size_t)grid * 8);
  k_fock_expand<<<grid, kFockBS, 0, s>>>(n_states, G.n_site, G.n_ops, G.stats, C.state.as<uint64_t>(),
                                         C.reps.as<uint64_t>(), C.stab.as<uint8_t>(), S.rowflag.as<uint8_t>(),
                                         C.perm_u8.as<uint8_t>(), S.phase.as<double2>(), dchi.as<double2>(),
                                         xpad.as<double2>(), atol, o, part.as<double>());
  SED_CUDA(cudaGetLastError());
  std::vector<double> hp(grid);
  SED_CUDA(cudaMemcpyAsync(hp.data(), part.p, (size_t)grid * 8, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
  double norm2 = 0.0;
  for (double v : hp) norm2 += v;
  if (norm2_out) *norm2_out = norm2;
  SED_REQUIRE(norm2 > atol, 1, "Expanded state has near-zero norm.");
  k_fock_scale<<<grid, kFockBS, 0, s>>>(n_states, o, 1.0 / std::sqrt(norm2));
  SED_CUDA(cudaGetLastError());
  if (!is_device)
    SED_CUDA(cudaMemcpyAsync(out, o, (size_t)n_states * 16, cudaMemcpyDeviceToHost, s));
  SED_CUDA(cudaStreamSynchronize(s));
}

}  // namespace sed
