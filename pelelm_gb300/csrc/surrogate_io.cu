// Loads a trained surrogate (".pgbs" file written by pelelm_gb300/surrogate_train.py) into
// device memory for the fused inference kernel (surrogate_kernel.cuh). No counterpart in the
// reference: the learned path is an addition behind the same reactor API.
//
// File layout (little endian):
//   char[8]  "PGBSURR1"
//   char[32] mechanism name (NUL padded)
//   int32[16] ns, nmodel, nlayer, n_in, k_half, k_in, n_out, n_out_pad, nel, split, 0...
//   int32[nlayer+1] layer widths (dims[0] = k_in, the padded split input)
//   int32[n_out] species of each output (-1 = temperature)
//   float64[n_in] x_mean, x_std, z_min, z_max (z = normalised feature range in training)
//   float64[n_out] y_scale
//   float64[nel*ns] A (element per gram of species), float64[ns*nel] P (least-norm projector)
//   float64[16] ood_margin, mis, cons, disT, disY, neg, tol_T, tol_Y, audit_frac, 0...
//   per member, per layer: float32 W (dims[l+1] x K_l, K_0 = k_half when split), float32 b
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "surrogate_host.h"

namespace pgb_host {

namespace {

uint16_t to_bf16(float f) {  // round to nearest even; NaN stays NaN
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x007FFFFFu)) return (uint16_t)((u >> 16) | 0x40u);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

struct Reader {
  FILE* f;
  bool ok = true;
  template <class T>
  void get(T* p, size_t n) {
    if (ok && n && std::fread(p, sizeof(T), n, f) != n) ok = false;
  }
};

}  // namespace

void sg_free(SgModel& m) {
  if (m.d_net) cudaFree(m.d_net);
  if (m.d_weights) cudaFree(m.d_weights);
  m = SgModel();
}

int sg_load(const char* path, const char* mech_name, int ns, const SgOverrides& ov, SgModel& out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_err("surrogate: cannot open '%s'", path);
  Reader rd{f};
  char magic[8], mech[33] = {0};
  int32_t hdr[16];
  rd.get(magic, 8);
  rd.get(mech, 32);
  rd.get(hdr, 16);
  if (!rd.ok || std::memcmp(magic, "PGBSURR1", 8) != 0) {
    std::fclose(f);
    return set_err("surrogate: '%s' is not a surrogate file", path);
  }
  const int fns = hdr[0], nmodel = hdr[1], nlayer = hdr[2], n_in = hdr[3], k_half = hdr[4], k_in = hdr[5];
  const int n_out = hdr[6], n_out_pad = hdr[7], nel = hdr[8], split = hdr[9];
  auto fail = [&](const char* why) {
    std::fclose(f);
    return set_err("surrogate '%s': %s", path, why);
  };
  if (std::strcmp(mech, mech_name) != 0) return fail("trained for another mechanism");
  if (fns != ns || n_in != 2 * ns + 2) return fail("species count does not match the mechanism");
  if (nmodel < 1 || nlayer < 2 || nlayer > pgb::SG_MAX_LAYERS || n_in > pgb::SG_MAX_IN) return fail("bad sizes");
  if (!split || k_half < n_in || k_in != 2 * k_half || k_in % 32 || k_in > pgb::SG_WIDTH)
    return fail("first layer must take the split input (k_in = 2 k_half, a multiple of 32, <= 256)");
  if (n_out < 1 || n_out > pgb::SG_NOUT_PAD || n_out_pad != pgb::SG_NOUT_PAD) return fail("bad output count");
  if (nel < 0 || nel > pgb::SG_MAX_EL) return fail("too many elements");
  std::vector<int32_t> dims(nlayer + 1), osp(n_out);
  rd.get(dims.data(), dims.size());
  rd.get(osp.data(), osp.size());
  if (!rd.ok) return fail("truncated");
  if (dims[0] != k_in || dims[nlayer] != n_out_pad) return fail("layer widths do not match the header");
  for (int l = 1; l < nlayer; ++l)
    if (dims[l] != pgb::SG_WIDTH) return fail("hidden layers must be 256 wide");
  for (int q = 0; q < n_out; ++q)
    if (osp[q] < -1 || osp[q] >= ns) return fail("bad output species index");
  std::vector<double> xm(n_in), xs(n_in), zmin(n_in), zmax(n_in), ys(n_out), A((size_t)nel * ns),
      Pm((size_t)ns * nel), gates(16);
  rd.get(xm.data(), n_in); rd.get(xs.data(), n_in); rd.get(zmin.data(), n_in); rd.get(zmax.data(), n_in);
  rd.get(ys.data(), n_out);
  rd.get(A.data(), A.size()); rd.get(Pm.data(), Pm.size());
  rd.get(gates.data(), 16);
  if (!rd.ok) return fail("truncated");
  const int use_models = std::min(nmodel, ov.models > 0 ? ov.models : pgb::SG_MAX_MODELS);

  // weights: BF16, first layer written twice (high and low input halves); 256-byte aligned blocks
  std::vector<size_t> woff, boff;
  size_t bytes = 0;
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  for (int m = 0; m < use_models; ++m)
    for (int l = 0; l < nlayer; ++l) {
      woff.push_back(bytes);
      bytes = align(bytes + (size_t)dims[l + 1] * dims[l] * 2);
      boff.push_back(bytes);
      bytes = align(bytes + (size_t)dims[l + 1] * 4);
    }
  std::vector<unsigned char> host(bytes, 0);
  for (int m = 0; m < nmodel; ++m)
    for (int l = 0; l < nlayer; ++l) {
      const int N = dims[l + 1], Kf = (l == 0) ? k_half : dims[l];
      std::vector<float> W((size_t)N * Kf), b(N);
      rd.get(W.data(), W.size());
      rd.get(b.data(), b.size());
      if (!rd.ok) return fail("truncated weights");
      if (m >= use_models) continue;
      const size_t idx = (size_t)m * nlayer + l;
      uint16_t* wd = reinterpret_cast<uint16_t*>(host.data() + woff[idx]);
      const int K = dims[l];
      for (int n = 0; n < N; ++n)
        for (int k = 0; k < Kf; ++k) {
          const uint16_t v = to_bf16(W[(size_t)n * Kf + k]);
          wd[(size_t)n * K + k] = v;
          if (l == 0) wd[(size_t)n * K + k_half + k] = v;
        }
      std::memcpy(host.data() + boff[idx], b.data(), (size_t)N * 4);
    }
  std::fclose(f);

  pgb::SurrogateNet net;
  std::memset(&net, 0, sizeof(net));
  net.nmodel = use_models;
  net.nlayer = nlayer;
  net.n_in = n_in;
  net.k_half = k_half;
  net.k_in = k_in;
  net.n_out = n_out;
  for (int l = 0; l <= nlayer; ++l) net.dims[l] = dims[l];
  const double margin = std::isnan(ov.ood_margin) ? gates[0] : ov.ood_margin;
  for (int q = 0; q < n_in; ++q) {
    if (!(xs[q] > 0.0)) return set_err("surrogate '%s': non-positive feature scale", path);
    net.x_mean[q] = (float)xm[q];
    net.x_inv_std[q] = (float)(1.0 / xs[q]);
    net.z_lo[q] = (float)(zmin[q] - margin);
    net.z_hi[q] = (float)(zmax[q] + margin);
  }
  for (int q = 0; q < n_out; ++q) {
    net.y_scale[q] = ys[q];
    net.out_species[q] = osp[q];
  }
  net.nel = nel;
  for (int e = 0; e < nel; ++e)
    for (int s = 0; s < ns; ++s) {
      net.A[e][s] = A[(size_t)e * ns + s];
      net.P[s][e] = Pm[(size_t)s * nel + e];
    }
  auto pick = [](double o, double file) { return std::isnan(o) ? file : o; };
  net.g_mis = pick(ov.mis, gates[1]);
  net.g_cons = pick(ov.cons, gates[2]);
  net.g_disT = pick(ov.disT, gates[3]);
  net.g_disY = pick(ov.disY, gates[4]);
  net.g_neg = pick(ov.neg, gates[5]);
  net.tol_T = pick(ov.tol_T, gates[6]);
  net.tol_Y = pick(ov.tol_Y, gates[7]);
  net.audit_frac = pick(ov.audit_frac, gates[8]);
  if (!(net.audit_frac >= 0.0 && net.audit_frac <= 1.0)) return set_err("surrogate: audit fraction must be in [0, 1]");

  SgModel m;
  PGB_CUDA(cudaMalloc(&m.d_weights, bytes));
  PGB_CUDA(cudaMemcpy(m.d_weights, host.data(), bytes, cudaMemcpyHostToDevice));
  for (int mm = 0; mm < use_models; ++mm)
    for (int l = 0; l < nlayer; ++l) {
      const size_t idx = (size_t)mm * nlayer + l;
      net.W[mm][l] = reinterpret_cast<const __nv_bfloat16*>(static_cast<unsigned char*>(m.d_weights) + woff[idx]);
      net.b[mm][l] = reinterpret_cast<const float*>(static_cast<unsigned char*>(m.d_weights) + boff[idx]);
    }
  if (cudaMalloc(&m.d_net, sizeof(net)) != cudaSuccess) {
    sg_free(m);
    return set_err("surrogate: out of device memory");
  }
  PGB_CUDA(cudaMemcpy(m.d_net, &net, sizeof(net), cudaMemcpyHostToDevice));
  m.audit_frac = net.audit_frac;
  m.nmodel = use_models;
  out = m;
  return 0;
}

}  // namespace pgb_host
