// Raw, layout-identical writer of the reference's integral and eigen datasets.
//
// The reference stores the orthogonalised, packed integrals of every k in
// setup-temp.hdf5 (hdf5SetupIntg.F90:86-222: groups
// /atomIntgGroup/{atomOverlap,atomKEOverlap,atomMVOverlap,atomNucOverlap}/%07d(k) and
// /atomIntgGroup/atomPotOverlap/%07d(k)/%07d(term), each a (2, n(n+1)/2)
// binary64 dataset) and the eigen-solutions in main-temp.hdf5
// (hdf5MainEval.f90:60-81: /eigenValues/%07d%07d(k, spin), (numStates);
// hdf5MainEvec.F90:81-119: /eigenVectors/real%07d%07d and imag%07d%07d,
// (valeDim, numStates)).  Without libhdf5 every dataset becomes
// <root>/<group>/<name>.bin holding its elements in the dataset's Fortran
// order as little-endian binary64, and <root>/manifest.json lists path, dims
// (Fortran order) and type of each, so that a converter (or h5py where it
// exists) rebuilds the HDF5 file one dataset at a time.
#include <cerrno>
#include <cstdio>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "olc_common.h"

namespace olc {

namespace {

// (row j, column i <= ...) upper part of a full [nk][nv][nv] matrix ->
// packed [nk][nv(nv+1)/2] complex, index j + i(i+1)/2 for j <= i.
__global__ void pack_upper_kernel(const double* __restrict__ full, int nv, int nk,
                                  double* __restrict__ packed) {
  const size_t plen = (size_t)nv * (nv + 1) / 2, total = plen * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / plen);
    const size_t r = idx % plen;
    int i = (int)((sqrt(8.0 * (double)r + 1.0) - 1.0) * 0.5);
    while ((size_t)i * (i + 1) / 2 > r) --i;
    while ((size_t)(i + 1) * (i + 2) / 2 <= r) ++i;
    const int j = (int)(r - (size_t)i * (i + 1) / 2);
    const size_t off = (size_t)k * nv * nv + (size_t)i * nv + j;
    packed[2 * idx] = full[2 * off];
    packed[2 * idx + 1] = full[2 * off + 1];
  }
}

std::string name7(int v) {
  char b[16];
  std::snprintf(b, sizeof b, "%07d", v);
  return b;
}

int make_dirs(const std::string& path) {
  for (size_t p = 1; p <= path.size(); ++p) {
    if (p == path.size() || path[p] == '/') {
      const std::string d = path.substr(0, p);
      if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST)
        return fail(OLC_ERR_ARG, "cannot create directory " + d);
    }
  }
  return OLC_OK;
}

struct Writer {
  std::string root;
  std::vector<std::string> entries;

  int dataset(const std::string& path, const std::vector<long long>& dims, const double* data) {
    const size_t slash = path.rfind('/');
    int st;
    if (slash != std::string::npos && (st = make_dirs(root + "/" + path.substr(0, slash)))) return st;
    size_t count = 1;
    for (long long d : dims) count *= (size_t)d;
    const std::string file = path + ".bin";
    FILE* f = std::fopen((root + "/" + file).c_str(), "wb");
    if (!f) return fail(OLC_ERR_ARG, "cannot open " + root + "/" + file);
    const size_t wrote = std::fwrite(data, sizeof(double), count, f);
    const int closed = std::fclose(f);
    if (wrote != count || closed != 0) return fail(OLC_ERR_ARG, "short write to " + file);
    std::string dj = "[";
    for (size_t q = 0; q < dims.size(); ++q) dj += (q ? ", " : "") + std::to_string(dims[q]);
    dj += "]";
    entries.push_back("    {\"path\": \"/" + path + "\", \"file\": \"" + file + "\", \"dims\": " + dj +
                      ", \"type\": \"float64\", \"order\": \"fortran\"}");
    return OLC_OK;
  }

  int finish(const std::string& kind) {
    FILE* f = std::fopen((root + "/manifest.json").c_str(), "wb");
    if (!f) return fail(OLC_ERR_ARG, "cannot open " + root + "/manifest.json");
    std::string s = "{\n  \"format\": \"olcao raw datasets\",\n  \"file\": \"" + kind + "\",\n  \"datasets\": [\n";
    for (size_t q = 0; q < entries.size(); ++q) s += entries[q] + (q + 1 < entries.size() ? ",\n" : "\n");
    s += "  ]\n}\n";
    const size_t wrote = std::fwrite(s.data(), 1, s.size(), f);
    const int closed = std::fclose(f);
    if (wrote != s.size() || closed != 0) return fail(OLC_ERR_ARG, "short write to manifest.json");
    return OLC_OK;
  }
};

}  // namespace

int write_setup_integrals(olc_context* ctx, const char* root) {
  if (!ctx->prepared || ctx->prep_form != OLC_FORM_STORED || !ctx->d_terms || !ctx->d_chol)
    return fail(OLC_ERR_ARG, "olc_write_setup_integrals: call olc_scf_prepare with OLC_FORM_STORED first");
  const int nv = ctx->dims.vale_dim, nk = ctx->dims.num_kpoints, pd = ctx->dims.pot_dim;
  const size_t plen = (size_t)ctx->dims.packed_len, plen2 = 2 * plen * nk;
  int st;
  if ((st = make_dirs(root))) return st;
  // overlap: pack the upper part of the orthogonalised S
  double* dS = nullptr;
  if ((st = cuda_check(ctx_malloc(ctx, (void**)&dS, 8 * plen2, ctx->stream), "malloc packed S"))) return st;
  pack_upper_kernel<<<(int)std::min<size_t>((plen * nk + 255) / 256, 152 * 16), 256, 0, ctx->stream>>>(
      ctx->d_chol, nv, nk, dS);
  count_launch();
  const int nfix = 2 + ctx->rel;
  std::vector<double> hS(plen2), hT(plen2 * (nfix + pd));
  st = cuda_check(cudaMemcpyAsync(hS.data(), dS, 8 * plen2, cudaMemcpyDeviceToHost, ctx->stream), "copy S");
  if (!st) st = cuda_check(cudaMemcpyAsync(hT.data(), ctx->d_terms, 8 * plen2 * (nfix + pd), cudaMemcpyDeviceToHost,
                                           ctx->stream), "copy terms");
  cudaFreeAsync(dS, ctx->stream);
  if (!st) st = cuda_check(cudaStreamSynchronize(ctx->stream), "write sync");
  if (st) return st;
  Writer w{root, {}};
  const std::vector<long long> dims = {2, (long long)plen};
  // stored terms: 0 = NP, 1 = KE, 2 = MV (rel = 1), then V_j
  for (int k = 0; k < nk; ++k) {
    const std::string kn = name7(k + 1);
    if ((st = w.dataset("atomIntgGroup/atomOverlap/" + kn, dims, hS.data() + 2 * plen * k))) return st;
    if ((st = w.dataset("atomIntgGroup/atomKEOverlap/" + kn, dims, hT.data() + plen2 + 2 * plen * k))) return st;
    if (ctx->rel &&
        (st = w.dataset("atomIntgGroup/atomMVOverlap/" + kn, dims, hT.data() + 2 * plen2 + 2 * plen * k))) return st;
    if ((st = w.dataset("atomIntgGroup/atomNucOverlap/" + kn, dims, hT.data() + 2 * plen * k))) return st;
    for (int j = 0; j < pd; ++j)
      if ((st = w.dataset("atomIntgGroup/atomPotOverlap/" + kn + "/" + name7(j + 1), dims,
                          hT.data() + (size_t)(nfix + j) * plen2 + 2 * plen * k))) return st;
  }
  return w.finish("setup-temp.hdf5");
}

int write_eigen(const char* root, int nk, int spin, int num_states, int vale_dim, const double* eig,
                const double* vectors) {
  int st;
  if ((st = make_dirs(root))) return st;
  Writer w{root, {}};
  std::vector<double> re((size_t)vale_dim * num_states), im(re.size());
  for (int k = 0; k < nk; ++k) {
    const std::string nm = name7(k + 1) + name7(spin);
    if ((st = w.dataset("eigenValues/" + nm, {num_states}, eig + (size_t)k * num_states))) return st;
    if (!vectors) continue;
    const double* v = vectors + 2 * (size_t)k * num_states * vale_dim;
    for (size_t e = 0; e < re.size(); ++e) {
      re[e] = v[2 * e];
      im[e] = v[2 * e + 1];
    }
    if ((st = w.dataset("eigenVectors/real" + nm, {vale_dim, num_states}, re.data()))) return st;
    if ((st = w.dataset("eigenVectors/imag" + nm, {vale_dim, num_states}, im.data()))) return st;
  }
  return w.finish("main-temp.hdf5");
}

}  // namespace olc
