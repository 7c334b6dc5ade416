// Leaf max-norm of one tree with its reduction scratch in static device
// memory: the same reduction as Forest::max_abs (the GPU form of
// a$D_tree_max_cc, src/m_aX_utils.f90:468-519), for callers that must not
// allocate. Its scratch is a file-scope __device__ array; its address is taken
// with cudaGetSymbolAddress once per device and context (again after a device
// reset), and every call clears what it uses with cudaMemsetAsync. Nothing here calls an allocating routine.
// Included at the end of solver.cu (one translation unit for the kernels).
#pragma once
#include <cstring>
#include <mutex>
#include <type_traits>

#include "forest.hpp"
#include "kernels.cuh"

namespace afv {

namespace {

constexpr int kStaticMaxTrees = 1024;

// Per-tree striped maxima, the per-tree reduced maxima and the one-tree mask:
// 1024 * 64 * 8 + 1024 * 8 + 1024 * 4 bytes = 536,576 bytes per device.
__device__ __align__(256) unsigned long long g_stripes[kStaticMaxTrees * dev::kStripes];
__device__ __align__(256) unsigned long long g_red[kStaticMaxTrees];
__device__ __align__(256) int g_mask[kStaticMaxTrees];

struct StaticScratch {
  unsigned long long* stripes = nullptr;
  unsigned long long* red = nullptr;
  int* mask = nullptr;
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
bool g_ready[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};
StaticScratch g_scratch[kMaxDevices];

// Unique id of the calling thread's current CUDA context (cuCtxGetId through
// the runtime's driver entry points, so the library links no driver library).
// A device reset or a rebuilt primary context gets a new id, and with it the
// module's static arrays may sit at new addresses.
int current_context_id(unsigned long long& id, std::string& err) {
  typedef int (*CtxGetCurrent)(void**);
  typedef int (*CtxGetId)(void*, unsigned long long*);
  static CtxGetCurrent get_current = nullptr;
  static CtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
        qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
      return err = "cuCtxGetCurrent / cuCtxGetId not available", AFV_ERR_CUDA;
    get_current = reinterpret_cast<CtxGetCurrent>(a);
    get_id = reinterpret_cast<CtxGetId>(b);
  }
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0)
    return err = "no current CUDA context", AFV_ERR_CUDA;
  return AFV_OK;
}

// Address of the static scratch in the current context (device `device` is
// current). Taken with cudaGetSymbolAddress the first time a context uses it
// and again whenever the context changes; the cached addresses serve every
// other call.
int static_scratch(int device, StaticScratch& out, std::string& err) {
  if (device < 0 || device >= kMaxDevices) return err = "device ordinal out of range", AFV_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long ctx = 0;
  if (int rc = current_context_id(ctx, err)) return rc;
  if (!g_ready[device] || g_ctx_id[device] != ctx) {
    StaticScratch s;
    cudaError_t e1 = cudaGetSymbolAddress((void**)&s.stripes, g_stripes);
    cudaError_t e2 = cudaGetSymbolAddress((void**)&s.red, g_red);
    cudaError_t e3 = cudaGetSymbolAddress((void**)&s.mask, g_mask);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
      cudaError_t e = e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3;
      return err = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e), AFV_ERR_CUDA;
    }
    g_scratch[device] = s;
    g_ctx_id[device] = ctx;
    g_ready[device] = true;
  }
  out = g_scratch[device];
  return AFV_OK;
}

template <class F>
bool with_leaf_nc(int D, int nc, F&& f) {
  using std::integral_constant;
  if (D == 2) {
    switch (nc) {
      case 2: f(integral_constant<int, 2>{}, integral_constant<int, 2>{}); return true;
      case 4: f(integral_constant<int, 2>{}, integral_constant<int, 4>{}); return true;
      case 8: f(integral_constant<int, 2>{}, integral_constant<int, 8>{}); return true;
      case 16: f(integral_constant<int, 2>{}, integral_constant<int, 16>{}); return true;
    }
  } else {
    switch (nc) {
      case 2: f(integral_constant<int, 3>{}, integral_constant<int, 2>{}); return true;
      case 4: f(integral_constant<int, 3>{}, integral_constant<int, 4>{}); return true;
      case 8: f(integral_constant<int, 3>{}, integral_constant<int, 8>{}); return true;
    }
  }
  return false;
}

}  // namespace

int Forest::max_abs_static(int t, int var, double* out, std::string& err) {
  if (t < 0 || t >= plan.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  if (var != AFV_PHI && var != AFV_RHS && var != AFV_TMP) return err = "unknown variable", AFV_ERR_INVALID;
  if (plan.n_trees > kStaticMaxTrees)
    return err = "forest has " + std::to_string(plan.n_trees) + " trees; the static-scratch norm takes at most " +
                 std::to_string(kStaticMaxTrees),
           AFV_ERR_INVALID;
  StaticScratch s;
  if (int rc = static_scratch(device, s, err)) return rc;
  const int nt = plan.n_trees;
  // Cleared every call: the stripes (maxima start at +0.0, whose bits are 0)
  // and the mask (only tree t set).
  cudaMemsetAsync(s.stripes, 0, sizeof(unsigned long long) * nt * dev::kStripes, stream);
  cudaMemsetAsync(s.mask, 0, sizeof(int) * nt, stream);
  cudaMemsetAsync(s.mask + t, 0x01, 1, stream);
  dev::Meta m;
  m.tree = meta.tree;
  m.parent = meta.parent;
  m.first_child = meta.first_child;
  m.offg = meta.offg;
  m.offi = meta.offi;
  m.bcval = meta.bcval;
  m.active = s.mask;
  m.desc = meta.desc;
  m.nbo2 = meta.nbo2;
  m.err = meta.err;
  m.wait_limit = meta.wait_limit;
  const double* v = var == AFV_PHI ? d64.phi : var == AFV_RHS ? d64.rhs : d64.tmp;
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
    int nl = n_leaves(l);
    if (!nl) continue;
    dev::BoxSet bs{leaves_list(l), 0, nl};
    with_leaf_nc(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
      constexpr int BPC = dev::kThreads / PER_BOX;
      long long groups = (nl + BPC - 1) / BPC;
      int grid = (int)std::max(1LL, std::min(groups, (long long)n_sm * 16));
      dev::k_maxabs<D, NC, double><<<grid, dev::kThreads, 0, stream>>>(m, bs, v, var != AFV_RHS, s.stripes);
    });
  }
  dev::k_stripe_reduce<<<(nt + 255) / 256, 256, 0, stream>>>(nt, s.stripes, s.red);
  unsigned long long bits = 0;
  cudaMemcpyAsync(&bits, s.red + t, sizeof(bits), cudaMemcpyDeviceToHost, stream);
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return err = std::string("max_abs_static: ") + cudaGetErrorString(e), AFV_ERR_CUDA;
  std::memcpy(out, &bits, sizeof(double));
  return check(err, "max_abs_static");
}

}  // namespace afv
