// Device forest and the FAS multigrid drivers: allocations, uploads, the
// kernel launches per level, and the V-cycle / FMG / solve schedules of
// src/m_aX_mg.f90, with all trees of the forest swept by each launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <utility>

#include "forest.hpp"
#include "kernels.cuh"
#include "coarse_end.cuh"

namespace afv {

// Forests of one process may live on several host threads (the request
// loop). Graph capture must not overlap calls that synchronise with the
// device or allocate pinned memory (forest creation and destruction), so
// those sections share one lock.
static std::mutex g_capture_mutex;

using dev::BoxSet;
using dev::Meta;
template <int N> using IC = std::integral_constant<int, N>;

// Calls f(IC<D>, IC<NC>) for the supported (dimension, block size) pairs.
template <class F>
static bool with_nc(int D, int nc, F&& f) {
  if (D == 2) {
    switch (nc) {
      case 2: f(IC<2>{}, IC<2>{}); return true;
      case 4: f(IC<2>{}, IC<4>{}); return true;
      case 8: f(IC<2>{}, IC<8>{}); return true;
      case 16: f(IC<2>{}, IC<16>{}); return true;
    }
  } else {
    switch (nc) {
      case 2: f(IC<3>{}, IC<2>{}); return true;
      case 4: f(IC<3>{}, IC<4>{}); return true;
      case 8: f(IC<3>{}, IC<8>{}); return true;
    }
  }
  return false;
}

static Meta meta_of(const DevMeta& d) {
  Meta m;
  m.tree = d.tree;
  m.parent = d.parent;
  m.first_child = d.first_child;
  m.offg = d.offg;
  m.offi = d.offi;
  m.bcval = d.bcval;
  m.active = d.active;
  m.desc = d.desc;
  m.nbo2 = d.nbo2;
  m.err = d.err;
  m.wait_limit = d.wait_limit;
  return m;
}

// Raises a kernel's dynamic shared-memory limit to smem on the current device
// and returns its resident blocks per SM (at least 1). The attribute is per
// device and the forests of a process may run on several devices and host
// threads, so the result is kept per (kernel, device) under a lock. (The
// shared-memory carve-out stays the driver's choice: forcing the largest one
// on every kernel shrinks L1 under the sweeps, whose neighbour loads use it,
// and made the C2 mixed solve 10% slower.)
struct KernelAttrs {
  const void* kern;
  int device, threads, smem, occ;
};
static int kernel_occupancy(const void* kern, int threads, int smem) {
  static std::mutex mu;
  static std::vector<KernelAttrs> known;
  int device = 0;
  cudaGetDevice(&device);
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& k : known)
    if (k.kern == kern && k.device == device && k.threads == threads && k.smem >= smem) return k.occ;
  // always: the 48 KB default counts the kernel's static shared memory too
  if (smem > 0) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
  occ = occ < 1 ? 1 : occ;
  known.push_back({kern, device, threads, smem, occ});
  return occ;
}

// Kernel launch with programmatic stream serialization: the next kernel on
// the stream may be scheduled while this one drains, and waits in
// dev::pdl_wait() for it to finish before touching memory.
template <class... KArgs, class... Args>
static void launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

static int grid_for(long long units, int n_sm) {
  long long cap = (long long)n_sm * 16;
  return (int)std::max(1LL, std::min(units, cap));
}

// Device allocations are stream-ordered (cudaMallocAsync / cudaFreeAsync on
// the forest's stream), so creating and destroying a forest does not
// synchronise the work of other forests on the device.
template <class T>
static int dmalloc(T** p, long long n, long long& bytes, cudaStream_t st) {
  size_t b = (size_t)std::max(1LL, n) * sizeof(T);
  if (cudaMallocAsync((void**)p, b, st) != cudaSuccess) {
    *p = nullptr;
    return AFV_ERR_NOMEM;
  }
  bytes += (long long)b;
  return AFV_OK;
}

template <class T>
static int dupload(T** p, const std::vector<T>& v, long long& bytes, cudaStream_t st) {
  int rc = dmalloc(p, (long long)v.size(), bytes, st);
  if (rc) return rc;
  if (!v.empty() &&
      cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return AFV_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? AFV_OK : AFV_ERR_CUDA;  // v may go away
}

// Freed device memory up to this size stays in the device's pool for the
// next forest instead of going back to the driver at every synchronisation.
static void retain_pool(int device) {
  static bool done[64] = {};
  if (device < 0 || device >= 64 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    unsigned long long keep = 8ULL << 30;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[device] = true;
}

Forest::~Forest() {
  std::lock_guard<std::mutex> lock(g_capture_mutex);
  cudaSetDevice(device);
  if (side) cudaStreamSynchronize(side);
  if (stream) cudaStreamSynchronize(stream);
  void* ptrs[] = {meta.parent, meta.first_child, meta.tree, meta.offg, meta.offi, meta.bcval,
                  meta.active, meta.desc, meta.nbo2, meta.err, meta.rmin, d64.phi, d64.rhs,
                  d64.tmp, d32.phi, d32.rhs, d32.tmp, base_phi64, base_rhs64, d_lists, d_norm, d_red,
                  d_fmax, d_count, d_failed, d_cycles, d_final, d_stage, d_stage_slots, d_solve_mask};
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, stream);
  for (double* p : xcc)
    if (p) cudaFreeAsync(p, stream);
  for (void* p : {(void*)fc, (void*)d_nb, (void*)d_lvl, (void*)d_qd, (void*)d_tags, (void*)d_ix, (void*)d_coef})
    if (p) cudaFreeAsync(p, stream);
  if (stream) cudaStreamSynchronize(stream);
  for (const ProfEntry& p : prof) {
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
  drop_graphs();
  for (void* p : {(void*)h_count, (void*)h_norm, (void*)h_cycles, (void*)h_final, (void*)h_failed, (void*)h_fmax,
                  (void*)h_solve_mask})
    if (p) cudaFreeHost(p);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (side) cudaStreamDestroy(side);
  if (loop_stream) cudaStreamDestroy(loop_stream);
  if (stream) cudaStreamDestroy(stream);
}

int Forest::check_device_error(std::string& err) {
  int h = 0;
  cudaMemcpyAsync(&h, meta.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
  cudaStreamSynchronize(stream);
  if (h) {
    cudaMemsetAsync(meta.err, 0, sizeof(int), stream);
    err = "a bounded device wait gave up (copy not completed in time)";
    return AFV_ERR_TIMEOUT;
  }
  return AFV_OK;
}

int Forest::check(std::string& err, const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return AFV_ERR_CUDA;
  }
  return AFV_OK;
}

cudaEvent_t Forest::prof_begin(int kind) {
  ++n_launches;
  if (!(prof_mask & (1 << kind))) return nullptr;
  if (group_on && kind == kProfSweep) return nullptr;  // timed by the group
  cudaEvent_t e;
  if (!event_pool.empty()) {
    e = event_pool.back();
    event_pool.pop_back();
  } else {
    cudaEventCreate(&e);
  }
  cudaEventRecord(e, stream);
  return e;
}

void Forest::prof_end(cudaEvent_t start, int kind, double b, int count) {
  if (group_on && kind == kProfSweep && count == 1) {
    group_bytes += b;
    ++group_count;
    return;
  }
  if (!start) return;
  cudaEvent_t e;
  if (!event_pool.empty()) {
    e = event_pool.back();
    event_pool.pop_back();
  } else {
    cudaEventCreate(&e);
  }
  cudaEventRecord(e, stream);
  prof.push_back(ProfEntry{start, e, kind, prof_level, b, count});
}

long long Forest::prof_entries(long long max, int* kind, int* level, double* ms, double* b, int* count) {
  cudaStreamSynchronize(stream);
  long long n = 0;
  for (const ProfEntry& p : prof) {
    if (n >= max) break;
    float x = 0;
    cudaEventElapsedTime(&x, p.start, p.stop);
    kind[n] = p.kind;
    level[n] = p.level;
    ms[n] = x;
    b[n] = p.bytes;
    count[n] = p.count;
    ++n;
  }
  return (long long)prof.size();
}

int Forest::prof_read(int kind, long long* launches, double* ms, double* b) {
  cudaStreamSynchronize(stream);
  long long n = 0;
  double t = 0, by = 0;
  for (const ProfEntry& p : prof) {
    if (p.kind != kind) continue;
    float x = 0;
    cudaEventElapsedTime(&x, p.start, p.stop);
    t += x;
    by += p.bytes;
    n += p.count;
  }
  *launches = n;
  *ms = t;
  *b = by;
  return AFV_OK;
}

void Forest::prof_reset() {
  cudaStreamSynchronize(stream);
  for (const ProfEntry& p : prof) {
    event_pool.push_back(p.start);
    event_pool.push_back(p.stop);
  }
  prof.clear();
}

// Brackets one launch with profiler events.
// One pair of events around consecutive half-sweeps of a level.
struct SweepGroup {
  Forest* f;
  cudaEvent_t e = nullptr;
  explicit SweepGroup(Forest* f_) : f(f_) {
    if (f->prof_mask & (1 << kProfSweep)) {
      e = f->prof_begin(kProfSweep);
      --f->n_launches;  // the group is not a launch
      f->group_on = true;
      f->group_bytes = 0;
      f->group_count = 0;
    }
  }
  ~SweepGroup() {
    if (e) {
      f->group_on = false;
      if (f->group_count)
        f->prof_end(e, kProfSweep, f->group_bytes, f->group_count);
      else
        f->prof_end(e, kProfSweep, 0.0, 0);
    }
  }
};

struct ProfScope {
  Forest* f;
  int kind;
  double bytes;
  cudaEvent_t e;
  ProfScope(Forest* f_, int k, double b) : f(f_), kind(k), bytes(b) { e = f->prof_begin(k); }
  ~ProfScope() { f->prof_end(e, kind, bytes); }
};

int Forest::create(const std::vector<const HostTree*>& trees, const afv_forest_opts* opts,
                   std::string& err) {
  std::lock_guard<std::mutex> lock(g_capture_mutex);
  int rc = build_plan(trees, plan, err);
  if (rc) return rc;
  device = opts ? opts->device : 0;
  mixed = opts ? opts->mixed_buffers != 0 : false;
  if (cudaSetDevice(device) != cudaSuccess) return err = "cudaSetDevice failed", AFV_ERR_CUDA;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&loop_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming) != cudaSuccess)
    return err = "cudaStreamCreate failed", AFV_ERR_CUDA;
  retain_pool(device);
  const Plan& p = plan;
  bytes = 0;
#define UP(field, vec) \
  if ((rc = dupload(&meta.field, p.vec, bytes, stream))) return err = "device allocation failed", rc;
  UP(parent, parent);
  UP(first_child, first_child);
  UP(tree, tree);
  UP(offg, offg);
  UP(offi, offi);
  UP(nbo2, nbo2);
  UP(rmin, r_min);
#undef UP
  if (dmalloc(&meta.err, 1, bytes, stream)) return err = "device allocation failed", AFV_ERR_NOMEM;
  cudaMemsetAsync(meta.err, 0, sizeof(int), stream);
  if ((rc = upload_bc(err))) return rc;
  std::vector<int> act(p.n_trees, 1);
  if ((rc = dupload(&meta.active, act, bytes, stream))) return err = "device allocation failed", rc;
  if ((rc = dupload(&d_solve_mask, act, bytes, stream))) return err = "device allocation failed", rc;
  host_active = act;

  if (dmalloc(&d64.phi, p.n_elem_g, bytes, stream) || dmalloc(&d64.tmp, p.n_elem_g, bytes, stream) ||
      dmalloc(&d64.rhs, p.n_elem_i, bytes, stream))
    return err = "device allocation of the FP64 state failed", AFV_ERR_NOMEM;
  cudaMemsetAsync(d64.phi, 0, p.n_elem_g * sizeof(double), stream);
  cudaMemsetAsync(d64.tmp, 0, p.n_elem_g * sizeof(double), stream);
  cudaMemsetAsync(d64.rhs, 0, p.n_elem_i * sizeof(double), stream);
  if (mixed) {
    if (dmalloc(&d32.phi, p.n_elem_g, bytes, stream) || dmalloc(&d32.tmp, p.n_elem_g, bytes, stream) ||
        dmalloc(&d32.rhs, p.n_elem_i, bytes, stream))
      return err = "device allocation of the FP32 state failed", AFV_ERR_NOMEM;
    cudaMemsetAsync(d32.phi, 0, p.n_elem_g * sizeof(float), stream);
    cudaMemsetAsync(d32.tmp, 0, p.n_elem_g * sizeof(float), stream);
    cudaMemsetAsync(d32.rhs, 0, p.n_elem_i * sizeof(float), stream);
    int l0 = p.min_lvl;
    long long ng = (long long)p.lvl_n[p.L(l0)] * (long long)std::pow(p.nc_at(l0) + 2, p.dim);
    long long ni = (long long)p.lvl_n[p.L(l0)] * (long long)std::pow(p.nc_at(l0), p.dim);
    if (dmalloc(&base_phi64, ng, bytes, stream) || dmalloc(&base_rhs64, ni, bytes, stream))
      return err = "device allocation failed", AFV_ERR_NOMEM;
  }
  // level lists
  std::vector<int> lists;
  int nlev = p.max_lvl - p.min_lvl + 1;
  leaves_off.assign(nlev, 0);
  parents_off.assign(nlev, 0);
  for (int k = 0; k < nlev; ++k) {
    leaves_off[k] = (int)lists.size();
    lists.insert(lists.end(), p.leaves[k].begin(), p.leaves[k].end());
    parents_off[k] = (int)lists.size();
    lists.insert(lists.end(), p.parents[k].begin(), p.parents[k].end());
  }
  all_leaves_off = (int)lists.size();
  lists.insert(lists.end(), p.all_leaves.begin(), p.all_leaves.end());
  if ((rc = dupload(&d_lists, lists, bytes, stream))) return err = "device allocation failed", rc;
  if (dmalloc(&d_norm, (long long)p.n_trees * dev::kStripes, bytes, stream) ||
      dmalloc(&d_red, p.n_trees, bytes, stream) || dmalloc(&d_fmax, p.n_trees, bytes, stream) ||
      dmalloc(&d_count, 4, bytes, stream) || dmalloc(&d_failed, p.n_trees, bytes, stream) ||
      dmalloc(&d_cycles, p.n_trees, bytes, stream) || dmalloc(&d_final, p.n_trees, bytes, stream))
    return err = "device allocation failed", AFV_ERR_NOMEM;
  cudaMemsetAsync(d_count, 0, 4 * sizeof(int), stream);
  if (cudaMallocHost((void**)&h_count, 4 * sizeof(int)) != cudaSuccess ||
      cudaMallocHost((void**)&h_norm, sizeof(unsigned long long) * p.n_trees) != cudaSuccess ||
      cudaMallocHost((void**)&h_cycles, sizeof(int) * p.n_trees) != cudaSuccess ||
      cudaMallocHost((void**)&h_final, sizeof(unsigned long long) * p.n_trees) != cudaSuccess ||
      cudaMallocHost((void**)&h_failed, sizeof(int) * p.n_trees) != cudaSuccess ||
      cudaMallocHost((void**)&h_fmax, sizeof(double) * p.n_trees) != cudaSuccess ||
      cudaMallocHost((void**)&h_solve_mask, sizeof(int) * p.n_trees) != cudaSuccess)
    return err = "pinned allocation failed", AFV_ERR_NOMEM;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return check(err, "forest create");
  return AFV_OK;
}

void Forest::drop_graphs() {
  for (auto& g : graphs)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
  graphs.clear();
}

// The FP32 correction of the trees in the run: one memset of the whole array,
// or per level the slots of the leading trees.
void Forest::zero_correction(cudaStream_t st) {
  if (!tree_limit) {
    cudaMemsetAsync(d32.phi, 0, sizeof(float) * plan.n_elem_g, st);
    return;
  }
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
    const int n = lvl_n(l);
    if (!n) continue;
    const int lo = plan.lvl_lo[plan.L(l)];
    const long long end = lo + n < plan.n_slots ? plan.offg[lo + n] : plan.n_elem_g;
    cudaMemsetAsync(d32.phi + plan.offg[lo], 0, sizeof(float) * (end - plan.offg[lo]), st);
  }
}

void Forest::norm_reset() {
  cudaMemsetAsync(d_norm, 0, sizeof(unsigned long long) * plan.n_trees * dev::kStripes, stream);
}

void Forest::norm_fold() {
  ProfScope ps(this, kProfOther, 8.0 * plan.n_trees * dev::kStripes);
  launch_k(dev::k_stripe_reduce, (plan.n_trees + 255) / 256, 256, 0, stream, plan.n_trees, d_norm, d_red);
}

int Forest::upload_bc(std::string& err) {
  long long b = 0;
  if (meta.bcval) cudaFreeAsync(meta.bcval, stream);
  meta.bcval = nullptr;
  if (dupload(&meta.bcval, plan.bcval, b, stream)) return err = "device allocation failed", AFV_ERR_NOMEM;
  if (!meta.desc && dmalloc(&meta.desc, (long long)plan.desc.size(), bytes, stream))
    return err = "device allocation failed", AFV_ERR_NOMEM;
  if (cudaMemcpyAsync(meta.desc, plan.desc.data(), plan.desc.size() * sizeof(SlotDesc),
                      cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return err = "descriptor upload failed", AFV_ERR_CUDA;
  return AFV_OK;
}

int Forest::set_active_all(int v) {
  std::vector<int> a(plan.n_trees, v);
  return set_active_host(a);
}

int Forest::set_active_host(const std::vector<int>& a) {
  host_active = a;
  cudaMemcpyAsync(meta.active, host_active.data(), sizeof(int) * a.size(), cudaMemcpyHostToDevice,
                  stream);
  cudaStreamSynchronize(stream);
  return AFV_OK;
}

// ---------------------------------------------------------------------------
// Host exchange
// ---------------------------------------------------------------------------


// Copies between the host layout and slot storage go level by level: the
// host buffer is the concatenation, over the tree's levels, of its boxes in
// level-list order. The per-tree sizes, the runs of boxes of one level and
// the slot orders on the device are made on the first exchange of a forest.
static int exchange_plan(Forest& F, std::string& err) {
  if (F.xfer_ready) return AFV_OK;
  const Plan& p = F.plan;
  const int D = p.dim;
  F.xfer_total.assign(p.n_trees, {0, 0});
  F.xfer_runs.assign(p.n_trees, {});
  F.xfer_order_off.assign(p.n_trees + 1, 0);
  std::vector<int> all;
  for (int t = 0; t < p.n_trees; ++t) {
    const std::vector<int>& order = p.host_order[t];
    F.xfer_order_off[t] = (long long)all.size();
    all.insert(all.end(), order.begin(), order.end());
    size_t i = 0;
    while (i < order.size()) {
      const int l = p.lvl[order[i]];
      size_t j = i;
      while (j < order.size() && p.lvl[order[j]] == l) ++j;
      long long si = 1, sg = 1;
      for (int d = 0; d < D; ++d) {
        si *= p.nc_at(l);
        sg *= p.nc_at(l) + 2;
      }
      F.xfer_runs[t].push_back({(int)i, (int)(j - i), l});
      F.xfer_total[t][0] += (long long)(j - i) * si;
      F.xfer_total[t][1] += (long long)(j - i) * sg;
      i = j;
    }
  }
  F.xfer_order_off[p.n_trees] = (long long)all.size();
  if (cudaMallocAsync((void**)&F.d_stage_slots, sizeof(int) * std::max<size_t>(1, all.size()), F.stream) !=
      cudaSuccess)
    return err = "staging allocation failed", AFV_ERR_NOMEM;
  cudaMemcpyAsync(F.d_stage_slots, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, F.stream);
  if (cudaStreamSynchronize(F.stream) != cudaSuccess) return F.check(err, "host exchange");
  F.xfer_ready = true;
  return AFV_OK;
}

static int exchange(Forest& F, int t, int var, double* host, int interior_only, bool to_dev,
                    std::string& err) {
  const Plan& p = F.plan;
  if (t < 0 || t >= p.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  if (var < AFV_PHI || var >= F.n_cc_vars()) return err = "unknown variable", AFV_ERR_INVALID;
  if (int rc = exchange_plan(F, err)) return rc;
  const int D = p.dim;
  const long long total = F.xfer_total[t][interior_only ? 0 : 1];
  // With zero_copy (the default), page-locked host memory, mapped into the
  // device's address space, is read or written by the scatter / gather
  // kernels directly, with no staging copy; those kernels then hold SMs for
  // the whole transfer. Otherwise (and for pageable memory) the bytes go
  // through a device staging buffer: one cudaMemcpyAsync on the copy engines
  // and a scatter / gather kernel at HBM speed, which leaves the SMs to other
  // work (another forest's solve) while the bytes cross the link.
  double* mapped = nullptr;
  if (F.zero_copy) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
        pa.devicePointer && pa.device == F.device)
      mapped = static_cast<double*>(pa.devicePointer);
    cudaGetLastError();  // an unregistered pointer is not an error here
  }
  if (!mapped && (F.stage_elems < total || !F.d_stage)) {
    if (F.d_stage) cudaFreeAsync(F.d_stage, F.stream);
    F.d_stage = nullptr;
    if (cudaMallocAsync((void**)&F.d_stage, sizeof(double) * std::max(1LL, total), F.stream) != cudaSuccess)
      return err = "staging allocation failed", AFV_ERR_NOMEM;
    F.stage_elems = total;
  }
  cudaStream_t st = F.stream;
  const int* slots = F.d_stage_slots + F.xfer_order_off[t];
  double* buf = mapped ? mapped : F.d_stage;
  if (to_dev && !mapped)
    cudaMemcpyAsync(F.d_stage, host, sizeof(double) * total, cudaMemcpyHostToDevice, st);
  Meta m = meta_of(F.meta);
  bool ghosted = var != AFV_RHS;
  double* dvar = F.var_ptr(var);
  long long off = 0;
  for (const Forest::XferRun& r : F.xfer_runs[t]) {
    const int nc = p.nc_at(r.lvl);
    long long per = 1;
    for (int d = 0; d < D; ++d) per *= interior_only ? nc : nc + 2;
    const int n = r.n;
    with_nc(D, nc, [&](auto d_, auto nc_) {
      constexpr int DD = decltype(d_)::value, NC = decltype(nc_)::value;
      int grid = grid_for((n * per + 255) / 256, F.n_sm);
      ProfScope ps(&F, kProfOther, 16.0 * n * per);
      if (to_dev)
        launch_k(dev::k_scatter<DD, NC, double>, grid, 256, 0, st, m, slots + r.first, n, buf + off, dvar,
                 interior_only, ghosted);
      else
        launch_k(dev::k_gather<DD, NC, double>, grid, 256, 0, st, m, slots + r.first, n, dvar, buf + off,
                 interior_only, ghosted);
    });
    off += n * per;
  }
  if (!to_dev && !mapped) cudaMemcpyAsync(host, F.d_stage, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return F.check(err, "host exchange");
  return F.check(err, "host exchange");
}

}  // namespace afv

namespace afv {

int forest_exchange_plan(Forest& F, std::string& err) { return exchange_plan(F, err); }

int forest_set_var(Forest& F, int t, int var, const double* host, int interior_only, std::string& err) {
  return exchange(F, t, var, const_cast<double*>(host), interior_only, true, err);
}
int forest_get_var(Forest& F, int t, int var, double* host, int interior_only, std::string& err) {
  return exchange(F, t, var, host, interior_only, false, err);
}

int Forest::get_var(int t, int var, double* host, int interior_only, std::string& err) {
  return forest_get_var(*this, t, var, host, interior_only, err);
}
int Forest::set_var(int t, int var, const double* host, int interior_only, std::string& err) {
  return forest_set_var(*this, t, var, host, interior_only, err);
}

// ---------------------------------------------------------------------------
// Level operators
// ---------------------------------------------------------------------------


// Launches the pipelined level kernel (sweep or ghost fill) on a box set.
template <int D, int NC, class T, int MODE>
static void launch_level(Forest& F, const Meta& m, BoxSet bs, T* phi, const T* rhs, int n, bool pull,
                         bool homog) {
  using C = dev::LevelCfg<D, NC, T, MODE>;
  const int occ = kernel_occupancy((const void*)dev::k_level_tma<D, NC, T, MODE>, dev::kThreads, (int)C::SMEM_B);
  const long long groups = (bs.n + C::BPC - 1) / C::BPC;
  const int grid = (int)std::max(1LL, std::min(groups, (long long)F.n_sm * occ));
  launch_k(dev::k_level_tma<D, NC, T, MODE>, grid, dev::kThreads, C::SMEM_B, F.stream, 
      m, bs, phi, rhs, n, pull ? 1 : 0, homog ? 1 : 0);
}

// Launches the warp-per-box sweep: W warps per block, S stages per warp.
template <int D, int NC, class T, int W, int S, int ASYNC>
static void launch_sweep_warp(Forest& F, const Meta& m, BoxSet bs, T* phi, const T* rhs, int n,
                              bool pull, bool homog) {
  using C = dev::WarpCfg<D, NC, T, W, S>;
  const int occ = kernel_occupancy((const void*)dev::k_sweep_warp<D, NC, T, W, S, ASYNC>, W * 32, (int)C::SMEM_B);
  // a level with fewer boxes than resident blocks gets one block per box
  const long long blocks = bs.n;
  const int grid = (int)std::max(1LL, std::min(blocks, (long long)F.n_sm * occ));
  launch_k(dev::k_sweep_warp<D, NC, T, W, S, ASYNC>, grid, W * 32, C::SMEM_B, F.stream, m, bs, phi, rhs, n, pull ? 1 : 0,
                                                                          homog ? 1 : 0);
}

// Launches the warp-per-parent correction (8 warps x 3 stages in FP32,
// 4 x 3 in FP64: about 195 KB of shared memory for 8^3 boxes).
template <int D, int NC, class T>
static void launch_correct_warp(Forest& F, const Meta& m, BoxSet bs, T* phi, T* tmp, bool pull, bool homog) {
  constexpr int W = std::is_same<T, float>::value ? 8 : 4, S = 3;
  using C = dev::CorrectCfg<D, NC, T, W, S>;
  auto go = [&](auto split_) {
    constexpr int SPLIT = decltype(split_)::value;
    auto kern = dev::k_correct_warp<D, NC, T, W, S, SPLIT>;
    const int occ = kernel_occupancy((const void*)kern, W * 32, (int)C::SMEM_B);
    const long long items = (long long)bs.n * (SPLIT == 2 ? C::FINE : 1);
    const long long blocks = items;  // one block per item when they are few
    const int grid = (int)std::max(1LL, std::min(blocks, (long long)F.n_sm * occ));
    launch_k(kern, grid, W * 32, (size_t)C::SMEM_B, F.stream, m, bs, phi, tmp, pull ? 1 : 0, homog ? 1 : 0);
  };
  // FP64: the prolongation (about 55 FP64 operations per parent cell) spread
  // over a warp per child, at the cost of a second launch (C2 FP64 solve
  // 28.73 ms against 28.86 ms with a warp per parent on levels of at least a
  // quarter as many parents as resident warps). FP32 keeps one launch (9.01
  // against 9.11 ms split).
  if constexpr (std::is_same<T, double>::value) {
    go(IC<1>{});
    go(IC<2>{});
    ++F.n_launches;  // the profiler scope around this call counts one
  } else {
    go(IC<0>{});
  }
}

dev_BoxSet Forest::level_set(int lvl) const {
  const int lo = plan.lvl_lo[plan.L(lvl)];
  return BoxSet{nullptr, lo, lvl_n(lvl), plan.offg[lo], plan.offi[lo]};
}

// Launches the warp-per-box restriction (16 warps x 3 stages in FP32,
// 8 x 3 in FP64: about 200 KB of shared memory, one block per SM).
template <int D, int NC, class T>
static void launch_restrict_warp(Forest& F, const Meta& m, BoxSet bs, T* phi, const T* rhs, T* tmp,
                                 bool homog) {
  constexpr int W = std::is_same<T, float>::value ? 16 : 8, S = 3;
  using C = dev::RestrictCfg<D, NC, T, W, S>;
  const int occ = kernel_occupancy((const void*)dev::k_restrict_warp<D, NC, T, W, S>, W * 32, (int)C::SMEM_B);
  // a level with fewer boxes than resident blocks gets one block per box
  const long long blocks = bs.n;
  const int grid = (int)std::max(1LL, std::min(blocks, (long long)F.n_sm * occ));
  launch_k(dev::k_restrict_warp<D, NC, T, W, S>, grid, W * 32, (size_t)C::SMEM_B, F.stream, m, bs, phi, rhs,
           tmp, homog ? 1 : 0);
}

// Launches the warp-per-box coarse right-hand side (same shape as the
// restriction).
template <int D, int NC, class T>
static void launch_coarse_warp(Forest& F, const Meta& m, BoxSet bs, T* phi, T* rhs, T* tmp, bool homog) {
  constexpr int W = std::is_same<T, float>::value ? 16 : 8, S = 3;
  using C = dev::CoarseCfg<D, NC, T, W, S>;
  const int occ = kernel_occupancy((const void*)dev::k_coarse_warp<D, NC, T, W, S>, W * 32, (int)C::SMEM_B);
  // a level with fewer boxes than resident blocks gets one block per box
  const long long blocks = bs.n;
  const int grid = (int)std::max(1LL, std::min(blocks, (long long)F.n_sm * occ));
  launch_k(dev::k_coarse_warp<D, NC, T, W, S>, grid, W * 32, (size_t)C::SMEM_B, F.stream, m, bs, phi, rhs, tmp,
           homog ? 1 : 0);
}

// Half-sweeps n_first .. n_first + n_count - 1 of a small level in one block
// (k_sweep_small); false if the level is too large for it.
template <class T>
bool Forest::sweeps_small(const Arrays<T>& a, int lvl, int n_first, int n_count, bool pull_first, bool homog) {
  const int nbx = lvl_n(lvl);
  if (!use_small_sweeps || nbx == 0) return false;
  bool done = false;
  with_nc(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    const size_t smem = (size_t)nbx * (sizeof(SlotDesc) + (G::SG + G::SI + G::NNB * G::NF) * sizeof(T) + 4 +
                                       4 * G::NNB);
    if (smem > (size_t)kSmallSmemBytes || (long long)nbx * G::SI > kSmallCells) return;
    kernel_occupancy((const void*)dev::k_sweep_small<D, NC, T>, dev::kSmallThreads, (int)kSmallSmemBytes);
    prof_level = lvl;
    ProfScope ps(this, kProfSweep, 3.0 * n_count * nbx * G::SI * sizeof(T));
    launch_k(dev::k_sweep_small<D, NC, T>, 1, dev::kSmallThreads, smem, stream, meta_of(meta), level_set(lvl), a.phi,
             (const T*)a.rhs, n_first, n_count, pull_first ? 1 : 0, homog ? 1 : 0);
    done = true;
  });
  return done;
}

template <class T>
void Forest::sweep(const Arrays<T>& a, int lvl, int n, bool pull, bool homog) {
  prof_level = lvl;
  int nbx = lvl_n(lvl);
  if (!nbx) return;
  BoxSet bs = level_set(lvl);
  Meta m = meta_of(meta);
  with_nc(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    // read phi and f, write phi over the interior
    ProfScope ps(this, kProfSweep, 3.0 * nbx * G::SI * sizeof(T));
    if (nbx <= direct_limit<T>() && (long long)nbx * (G::SI / 2) <= (1LL << 24)) {
      const long long items = (long long)nbx * (G::SI / 2);
      launch_k(dev::k_sweep_direct<D, NC, T>, (int)((items + 255) / 256), 256, 0, stream, m, bs, a.phi,
               (const T*)a.rhs, n, pull ? 1 : 0, homog ? 1 : 0);
    } else if (sweep_kernel == 0) {
      launch_level<D, NC, T, dev::kModeSweep>(*this, m, bs, a.phi, a.rhs, n, pull, homog);
    } else if constexpr (std::is_same<T, float>::value) {
      switch (sweep_kernel) {
        case 1: launch_sweep_warp<D, NC, T, 16, 3, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        case 2: launch_sweep_warp<D, NC, T, 16, 3, 1>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        case 3: launch_sweep_warp<D, NC, T, 16, 2, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        case 4: launch_sweep_warp<D, NC, T, 12, 3, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        default: launch_sweep_warp<D, NC, T, 24, 2, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
      }
    } else {
      // FP64: 6 warps x 3 stages by default (2.6 % faster FP64 solves on C2 than 8 x 3)
      switch (sweep_kernel) {
        case 1: launch_sweep_warp<D, NC, T, 6, 3, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        case 2: launch_sweep_warp<D, NC, T, 8, 3, 1>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        case 3: launch_sweep_warp<D, NC, T, 8, 2, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        case 4: launch_sweep_warp<D, NC, T, 8, 3, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
        default: launch_sweep_warp<D, NC, T, 12, 2, 0>(*this, m, bs, a.phi, a.rhs, n, pull, homog); break;
      }
    }
  });
}

template <class T>
void Forest::fill(const Arrays<T>& a, int lvl, bool homog) {
  int nbx = lvl_n(lvl);
  if (!nbx) return;
  fill_set(a, lvl, level_set(lvl), homog);
}

template <class T>
void Forest::fill_set(const Arrays<T>& a, int lvl, BoxSet bs, bool homog) {
  prof_level = lvl;
  if (!bs.n) return;
  Meta m = meta_of(meta);
  with_nc(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    // read the neighbour face value, write the ghost value
    ProfScope ps(this, kProfFill, 2.0 * bs.n * G::NNB * G::NF * sizeof(T));
    launch_level<D, NC, T, dev::kModeFill>(*this, m, bs, a.phi, nullptr, 0, true, homog);
  });
}

template <class T>
void Forest::restrict_res(const Arrays<T>& a, int lvl, bool with_res, bool pull, bool homog) {
  prof_level = lvl;
  int nbx = lvl_n(lvl);
  if (!nbx || lvl <= plan.min_lvl) return;
  BoxSet bs = level_set(lvl);
  Meta m = meta_of(meta);
  bool sub = lvl <= 1;
  with_nc(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    constexpr int H = NC / 2;
    constexpr int PER_BOX = D == 2 ? H * H : H * H * H;
    constexpr int BPC = dev::boxes_per_cta<G::SG, PER_BOX, T>(1);
    int grid = grid_for((nbx + BPC - 1) / BPC, n_sm);
    // read phi, f; write the parent's phi and tmp (2 values per 2^D fine cells)
    ProfScope ps(this, kProfRestrict,
                 (2.0 + 2.0 / (1 << D)) * nbx * G::SI * sizeof(T));
    if (!with_res) {
      // phi alone: one thread per parent cell, no staging
      constexpr int PAR = D == 2 ? H * H : H * H * H;
      const int g2 = grid_for(((long long)nbx * PAR + dev::kThreads - 1) / dev::kThreads, n_sm);
      if (sub)
        launch_k(dev::k_restrict_phi<D, NC, true, T>, g2, dev::kThreads, 0, stream, m, bs, a.phi);
      else
        launch_k(dev::k_restrict_phi<D, NC, false, T>, g2, dev::kThreads, 0, stream, m, bs, a.phi);
    } else if (sub)
      launch_k(dev::k_restrict_res<D, NC, true, T>, grid, dev::kThreads, 0, stream, 
          m, bs, a.phi, a.rhs, a.tmp, with_res ? 1 : 0, pull ? 1 : 0, homog ? 1 : 0);
    else if (with_res && pull && use_restrict_warp)
      launch_restrict_warp<D, NC, T>(*this, m, bs, a.phi, a.rhs, a.tmp, homog);
    else
      launch_k(dev::k_restrict_res<D, NC, false, T>, grid, dev::kThreads, 0, stream, 
          m, bs, a.phi, a.rhs, a.tmp, with_res ? 1 : 0, pull ? 1 : 0, homog ? 1 : 0);
  });
}

template <class T>
void Forest::coarse_rhs(const Arrays<T>& a, int lp, bool copy_tmp, bool pull, bool homog) {
  prof_level = lp;
  int np = n_parents(lp);
  if (!np) return;
  BoxSet bs{parents_list(lp), 0, np};
  Meta m = meta_of(meta);
  with_nc(plan.dim, plan.nc_at(lp), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
    constexpr int BPC = dev::boxes_per_cta<G::SG, PER_BOX, T>(1);
    int grid = grid_for((np + BPC - 1) / BPC, n_sm);
    // read phi, tmp; write rhs, tmp
    ProfScope ps(this, kProfCoarseRhs, 4.0 * np * G::SI * sizeof(T));
    if (copy_tmp && pull && use_restrict_warp && lp >= 1)
      launch_coarse_warp<D, NC, T>(*this, m, bs, a.phi, a.rhs, a.tmp, homog);
    else
      launch_k(dev::k_coarse_rhs<D, NC, T>, grid, dev::kThreads, 0, stream, 
          m, bs, a.phi, a.rhs, a.tmp, copy_tmp ? 1 : 0, pull ? 1 : 0, homog ? 1 : 0);
  });
}

template <class T>
void Forest::correct(const Arrays<T>& a, int lp, bool pull, bool homog) {
  prof_level = lp;
  int np = n_parents(lp);
  if (!np) return;
  BoxSet bs{parents_list(lp), 0, np};
  Meta m = meta_of(meta);
  bool sub = lp + 1 <= 1;
  with_nc(plan.dim, plan.nc_at(lp), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
    constexpr int BPC = dev::boxes_per_cta<G::SG, PER_BOX, T>(1);
    int grid = grid_for((np + BPC - 1) / BPC, n_sm);
    // parent: read phi, tmp, write tmp; children: read and write phi
    ProfScope ps(this, kProfCorrect, (3.0 + 2.0 * (1 << D)) * np * G::SI * sizeof(T));
    const int pl = pull ? 1 : 0, hg = homog ? 1 : 0;
    if (sub) {
      if constexpr (!(D == 2 && NC == 16) && !(D == 3 && NC == 8))
        launch_k(dev::k_correct<D, NC, true, T>, grid, dev::kThreads, 0, stream, m, bs, a.phi, a.tmp, pl, hg);
    } else if (use_restrict_warp) {
      launch_correct_warp<D, NC, T>(*this, m, bs, a.phi, a.tmp, pull, homog);
    } else {
      launch_k(dev::k_correct<D, NC, false, T>, grid, dev::kThreads, 0, stream, m, bs, a.phi, a.tmp, pl, hg);
    }
  });
}

template <class T>
void Forest::residual(const Arrays<T>& a, int lvl, unsigned long long* norm, bool store) {
  prof_level = lvl;
  int nbx = lvl_n(lvl);
  if (!nbx) return;
  BoxSet bs = level_set(lvl);
  Meta m = meta_of(meta);
  with_nc(plan.dim, plan.nc_at(lvl), [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
    constexpr int BPC = dev::kThreads / PER_BOX;
    int grid = grid_for((nbx + BPC - 1) / BPC, n_sm);
    ProfScope ps(this, kProfResidual, (store ? 3.0 : 2.0) * nbx * G::SI * sizeof(T));
    launch_k(dev::k_residual<D, NC, T>, grid, dev::kThreads, 0, stream, m, bs, a.phi, a.rhs, a.tmp, norm,
                                                                 store ? 1 : 0);
  });
}

// gsrb_boxes, src/m_aX_mg.f90:397-420: 2*n_cycle half-sweeps, each followed by
// a ghost fill. The fill after half-sweep n is folded into half-sweep n+1
// (pull); the last one is a separate launch.
template <class T>
void Forest::gsrb_boxes(const Arrays<T>& a, int lvl, int n_cycle, bool homog) {
  if (!lvl_n(lvl) || n_cycle <= 0) return;
  for (int n = 1; n <= 2 * n_cycle; ++n) sweep(a, lvl, n, n > 1, homog);
  fill(a, lvl, homog);
}

// update_coarse (copy_tmp) and set_coarse_phi_rhs (no copy),
// src/m_aX_mg.f90:424-517.
template <class T>
void Forest::update_coarse_t(const Arrays<T>& a, int lvl, bool homog, bool copy_tmp) {
  restrict_res(a, lvl, true);
  fill(a, lvl - 1, homog);
  coarse_rhs(a, lvl - 1, copy_tmp);
}

// mg$D_fas_vcycle, src/m_aX_mg.f90:208-255 (without the residual branch).
// The reference's ghost fills are folded into the kernels that follow them:
// a half-sweep pulls the ghosts its colour needs, the restriction pulls the
// fine level's ghosts, and the coarse right-hand side pulls (and stores) the
// ghosts of the parents after restriction. Each of these reads the same values
// the reference's fill would have stored, so results are unchanged. Only the
// first half-sweep on the top level reads stored ghosts (valid on input), and
// every level ends the cycle with a stored ghost fill (valid on output).
// base64: smooth the coarsest level in FP64 (mixed cycle).
// Launches k_coarse_end: one block per tree over the nl levels 1 .. 2 - nl.
void Forest::coarse_end(const Arrays<float>& a, const MgOpts& mg, int nl) {
  prof_level = 1;
  dev::CeSlots sl{};
  for (int L = 0; L < nl; ++L) sl.lo[L] = plan.lvl_lo[plan.L(1 - L)];
  Meta m = meta_of(meta);
  with_nc(plan.dim, plan.nc, [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    ProfScope ps(this, kProfCoarseEnd, 4.0 * (G::SG + 2 * G::SI) * n_trees_run());
    auto go = [&](auto nl_) {
      constexpr int NL = decltype(nl_)::value;
      if constexpr ((NC >> (NL - 1)) >= 2)
        launch_k(dev::k_coarse_end<D, NC, NL>, n_trees_run(), dev::kCoarseEndThreads, 0, stream, m, sl, a.phi,
                 (const float*)a.rhs, mg.n_down, mg.n_up, mg.n_base);
    };
    switch (nl) {
      case 1: go(IC<1>{}); break;
      case 2: go(IC<2>{}); break;
      case 3: go(IC<3>{}); break;
      default: go(IC<4>{}); break;
    }
  });
}

// Levels l0..1 run by k_coarse_end (0: not eligible): every tree has one box
// on each of them, in tree order, with no refinement boundary and periodic
// faces only onto the box itself; at most four levels, each with at least 2
// cells per side.
int Forest::coarse_end_depth(int highest) {
  if (!use_coarse_end || highest < 2 || plan.min_lvl > 1) return 0;
  if (coarse_end_levels >= 0) return coarse_end_levels;
  const Plan& p = plan;
  const int nl = 2 - p.min_lvl;
  int ok = nl <= dev::kCoarseEndMaxLevels && (p.nc >> (nl - 1)) >= 2;
  const int NNB = 2 * p.dim;
  for (int l = p.min_lvl; ok && l <= 1; ++l) {
    if (p.lvl_n[p.L(l)] != p.n_trees || p.nc_at(l) != (p.nc >> (1 - l))) ok = 0;
    for (int t = 0; ok && t < p.n_trees; ++t) {
      const int sl = p.lvl_lo[p.L(l)] + t;
      if (p.tree[sl] != t) ok = 0;
      for (int f = 0; ok && f < NNB; ++f) {
        const SlotDesc& d = p.desc[sl];
        if (d.code[f] == kFaceRefinement || (d.code[f] >= 0 && d.nbo[f] != p.offg[sl])) ok = 0;
      }
    }
  }
  coarse_end_levels = ok ? nl : 0;
  return coarse_end_levels;
}

template <class T>
void Forest::vcycle_t(const Arrays<T>& a, const MgOpts& mg, int highest, bool homog, bool base64,
                      bool inner) {
  const int l0 = plan.min_lvl;
  auto sweeps = [&](const auto& arr, int l, int n_cycle) {
    if (n_cycle <= 0) return;
    SweepGroup sg(this);
    if (sweeps_small(arr, l, 1, 2 * n_cycle, l != highest, homog)) return;
    for (int n = 1; n <= 2 * n_cycle; ++n) sweep(arr, l, n, n > 1 || l != highest, homog);
  };
  // The correction cycle's coarse end (levels l0..1) in one launch.
  const int ce = (std::is_same<T, float>::value && inner && homog && base64) ? coarse_end_depth(highest) : 0;
  const int l_low = ce ? 2 : l0 + 1;
  for (int l = highest; l >= l_low; --l) {
    sweeps(a, l, mg.n_down);
    restrict_res(a, l, true, true, homog);
    coarse_rhs(a, l - 1, true, true, homog);
  }
  if (ce) {
    if constexpr (std::is_same<T, float>::value) coarse_end(a, mg, ce);
  } else if (base64 && !std::is_same<T, double>::value) {
    long long ng = 0, ni = 0;
    int nb0 = lvl_n(l0);
    ng = (long long)nb0 * (long long)std::pow(plan.nc_at(l0) + 2, plan.dim);
    ni = (long long)nb0 * (long long)std::pow(plan.nc_at(l0), plan.dim);
    int g1 = grid_for((ng + 255) / 256, n_sm), g2 = grid_for((ni + 255) / 256, n_sm);
    {
      ProfScope ps(this, kProfOther, (8.0 + sizeof(T)) * ng);
      launch_k(dev::k_convert<double, T>, g1, 256, 0, stream, base_phi64, a.phi, ng);
    }
    {
      ProfScope ps(this, kProfOther, (8.0 + sizeof(T)) * ni);
      launch_k(dev::k_convert<double, T>, g2, 256, 0, stream, base_rhs64, a.rhs, ni);
    }
    Arrays<double> b{base_phi64, base_rhs64, nullptr};
    if (mg.n_base > 0) {
      sweeps(b, l0, mg.n_base);
      fill(b, l0, homog);
    }
    {
      ProfScope ps(this, kProfOther, (8.0 + sizeof(T)) * ng);
      launch_k(dev::k_convert<T, double>, g1, 256, 0, stream, a.phi, base_phi64, ng);
    }
  } else if (mg.n_base > 0) {
    sweeps(a, l0, mg.n_base);
    fill(a, l0, homog);
  }
  for (int l = l_low; l <= highest; ++l) {
    // Inner correction cycle of the mixed path: its result is read only on
    // interiors, and its ghost cells only on parents (by the correction of
    // their children and by the children's refinement-boundary ghosts), so
    // the ghost fill of level l-1 is done by the correction itself, on the
    // parents only. The FP64 cycle fills every box, as the reference does.
    correct(a, l - 1, inner && l - 1 > l0, homog);
    if (mg.n_up > 0) {
      SweepGroup sg(this);
      if (!sweeps_small(a, l, 1, 2 * mg.n_up, true, homog))
        for (int n = 1; n <= 2 * mg.n_up; ++n) sweep(a, l, n, true, homog);
    }
    if (!inner) fill(a, l, homog);
  }
}

// ---------------------------------------------------------------------------
// FP64 entry points
// ---------------------------------------------------------------------------

void Forest::fill64(int lvl) { fill(d64, lvl, false); }

int Forest::gsrb_level(int lvl, int n_cycle, std::string& err) {
  if (generic()) {
    gen_coef();
    gen_gsrb_boxes(lvl, n_cycle);
    if (int rc = check(err, "gsrb_level")) return rc;
    return check_device_error(err);
  }
  gsrb_boxes(d64, lvl, n_cycle, false);
  if (int rc = check(err, "gsrb_level")) return rc;
  return check_device_error(err);
}
int Forest::fill_level(int lvl, std::string& err) {
  fill(d64, lvl, false);
  return check(err, "fill_level");
}
int Forest::update_coarse(int lvl, std::string& err) {
  if (lvl <= plan.min_lvl || lvl > plan.max_lvl) return err = "level out of range", AFV_ERR_INVALID;
  if (generic()) {
    gen_coef();
    gen_update_coarse(lvl, true);
  } else {
    update_coarse_t(d64, lvl, false, true);
  }
  return check(err, "update_coarse");
}
int Forest::correct_children(int lp, std::string& err) {
  if (lp < plan.min_lvl || lp >= plan.max_lvl) return err = "level out of range", AFV_ERR_INVALID;
  if (generic())
    gen_correct(lp);
  else
    correct(d64, lp);
  return check(err, "correct_children");
}
int Forest::residual_all(unsigned long long* norm, std::string& err) {
  if (generic()) gen_coef();
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l)
    if (generic())
      gen_residual(l, norm);
    else
      residual(d64, l, norm, true);
  return check(err, "residual");
}

int Forest::vcycle(const MgOpts& mg, int highest, bool set_residual, std::string& err) {
  if (highest < plan.min_lvl) return err = "highest_lvl below the coarsest level", AFV_ERR_INVALID;
  highest = std::min(highest, plan.max_lvl);
  if (generic()) {
    gen_coef();
    gen_vcycle(mg, highest, set_residual);
  } else {
    vcycle_t(d64, mg, highest, false, false);
    if (set_residual)
      for (int l = plan.min_lvl; l <= highest; ++l) residual(d64, l, nullptr, true);
  }
  if (int rc = check(err, "vcycle")) return rc;
  return check_device_error(err);
}

// Times the kernel variants on this forest (FP32 correction V-cycles on the
// mixed scratch state, which every solve re-initialises) and keeps the
// fastest: first the sweep kernel (block-pipelined, warp-per-box with bulk
// copies in four warp / stage shapes, warp-per-box with per-lane copies),
// then, with it, the small-level sweep fusion and the one-launch coarse end
// (both on / off). Needs the mixed buffers. ms receives the ms per V-cycle of
// sweep kernels 0..5, then of the four (small sweeps, coarse end) settings
// (0,0), (0,1), (1,0), (1,1).
int Forest::autotune_all(int* sweep_out, int* small_out, int* coarse_out, float* ms_out, std::string& err) {
  if (!mixed) return err = "autotune needs a forest created with mixed_buffers", AFV_ERR_STATE;
  MgOpts mg;
  mg.n_down = mg.n_up = mg.n_base = 2;
  const int saved_mask = prof_mask;
  prof_mask = 0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_cycles = [&]() -> float {
    vcycle_t(d32, mg, plan.max_lvl, true, true, true);  // warm-up (first launches set attributes)
    cudaEventRecord(e0, stream);
    for (int r = 0; r < 3; ++r) vcycle_t(d32, mg, plan.max_lvl, true, true, true);
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / 3;
  };
  float best_ms = 1e30f;
  int best = sweep_kernel;
  for (int c = 0; c <= 5; ++c) {
    sweep_kernel = c;
    const float ms = time_cycles();
    if (ms_out) ms_out[c] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  sweep_kernel = best;
  bool best_small = use_small_sweeps, best_ce = use_coarse_end;
  best_ms = 1e30f;
  for (int k = 0; k < 4; ++k) {
    use_small_sweeps = (k >> 1) & 1;
    use_coarse_end = k & 1;
    coarse_end_levels = -1;
    const float ms = time_cycles();
    if (ms_out) ms_out[6 + k] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best_small = use_small_sweeps;
      best_ce = use_coarse_end;
    }
  }
  use_small_sweeps = best_small;
  use_coarse_end = best_ce;
  coarse_end_levels = -1;
  tune_defect(e0, e1, nullptr);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  prof_mask = saved_mask;
  drop_graphs();
  if (sweep_out) *sweep_out = sweep_kernel;
  if (small_out) *small_out = use_small_sweeps ? 1 : 0;
  if (coarse_out) *coarse_out = use_coarse_end ? 1 : 0;
  if (int rc = check(err, "autotune")) return rc;
  return check_device_error(err);
}

// The fixed-point defect's cells per thread, 1, 2 and 4 (those that exist
// for the forest's box shape; ms3[k] = -1 for the others): five launches of
// each alone, timed between e0 and e1 on the forest's stream; the fastest is
// kept. The defect writes only the correction's right-hand side and the
// norms, which every solve recomputes.
void Forest::tune_defect(cudaEvent_t e0, cudaEvent_t e1, float* ms3) {
  const int cands[3] = {1, 2, 4};
  for (int k = 0; k < 3; ++k)
    if (ms3) ms3[k] = -1.f;
  if (!defect_fx || n_all_leaves() == 0) return;
  const int shapes = defect_shapes();
  const int saved_mask = prof_mask;
  prof_mask = 0;
  float best_ms = 1e30f;
  int best = defect_cells;
  for (int k = 0; k < 3; ++k) {
    if (!(shapes & cands[k])) continue;
    defect_cells = cands[k];
    norm_reset();
    launch_defect();  // warm-up
    cudaEventRecord(e0, stream);
    for (int r = 0; r < 5; ++r) {
      norm_reset();
      launch_defect();
    }
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms3) ms3[k] = ms / 5;
    if (ms < best_ms) {
      best_ms = ms;
      best = cands[k];
    }
  }
  defect_cells = best;
  prof_mask = saved_mask;
  drop_graphs();
}

int Forest::autotune_defect(int* cells, float* ms3, std::string& err) {
  if (!mixed) return err = "autotune needs a forest created with mixed_buffers", AFV_ERR_STATE;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  tune_defect(e0, e1, ms3);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cells) *cells = defect_cells;
  if (int rc = check(err, "autotune_defect")) return rc;
  return check_device_error(err);
}

// The sweep kernel alone (the first part of autotune_all): variants 1, 2, 0.
int Forest::autotune(int* choice, float* ms_out, std::string& err) {
  if (!mixed) return err = "autotune needs a forest created with mixed_buffers", AFV_ERR_STATE;
  float ms[10];
  const bool small = use_small_sweeps, ce = use_coarse_end;
  const int dc = defect_cells;
  int rc = autotune_all(choice, nullptr, nullptr, ms, err);
  use_small_sweeps = small;  // this entry point tunes the sweep kernel only
  use_coarse_end = ce;
  defect_cells = dc;
  coarse_end_levels = -1;
  if (ms_out) {
    ms_out[0] = ms[1];
    ms_out[1] = ms[2];
    ms_out[2] = ms[0];
  }
  if (!rc && choice && *choice > 2) {  // keep the documented choice among 0..2
    int c = 1;
    for (int k : {0, 2})
      if (ms[k] < ms[c]) c = k;
    sweep_kernel = c;
    *choice = c;
  }
  drop_graphs();
  return rc;
}

// rhs of one tree := sum of Gaussians (or their Laplacian) at the cell
// centres, evaluated on the device: one launch per level over the tree's
// slots of that level (a contiguous range, trees being stored tree-major
// within a level).
int Forest::set_source_device(int t, int lpl, int n_gauss, const double* gauss, std::string& err) {
  if (t < 0 || t >= plan.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  if (n_gauss < 0 || n_gauss > dev::kMaxGauss)
    return err = "at most " + std::to_string(dev::kMaxGauss) + " Gaussians on the device", AFV_ERR_INVALID;
  dev::GaussSet gs;
  gs.n = n_gauss;
  gs.lpl = lpl;
  for (int k = 0; k < n_gauss * (2 + plan.dim); ++k) gs.g[k] = gauss[k];
  Meta m = meta_of(meta);
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
    const auto [a, b] = tree_level_range(t, l);
    if (a < 0) continue;
    BoxSet bs{nullptr, a, b - a + 1, plan.offg[a], plan.offi[a]};
    with_nc(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      long long items = (long long)bs.n * G::SI;
      ProfScope ps(this, kProfOther, 8.0 * items);
      launch_k(dev::k_source<D, NC>, grid_for(bs.n, n_sm), dev::kThreads, 0, stream, m, bs, t,
               (const double*)meta.rmin, gs, d64.rhs);
    });
  }
  return check(err, "set_source_device");
}

// cc(..., var) := 0 on every box of one tree, ghost cells included (a
// tree's boxes of one level are consecutive slots).
std::pair<int, int> Forest::tree_level_range(int t, int l) {
  const int nlev = plan.max_lvl - plan.min_lvl + 1;
  if (tl_first.empty()) {
    tl_first.assign((size_t)plan.n_trees * nlev, -1);
    tl_last.assign((size_t)plan.n_trees * nlev, -1);
    for (int ll = plan.min_lvl; ll <= plan.max_lvl; ++ll) {
      const int lo = plan.lvl_lo[plan.L(ll)], n = plan.lvl_n[plan.L(ll)];
      for (int k = 0; k < n; ++k) {
        const size_t i = (size_t)plan.tree[lo + k] * nlev + (ll - plan.min_lvl);
        if (tl_first[i] < 0) tl_first[i] = lo + k;
        tl_last[i] = lo + k;
      }
    }
  }
  if (l < plan.min_lvl || l > plan.max_lvl) return {-1, -1};
  const size_t i = (size_t)t * nlev + (l - plan.min_lvl);
  return {tl_first[i], tl_last[i]};
}

int Forest::zero_tree(int t, int var, std::string& err) {
  if (t < 0 || t >= plan.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  double* v = var_ptr(var);
  if (!v) return err = "unknown variable", AFV_ERR_INVALID;
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
    const auto [a, b] = tree_level_range(t, l);
    if (a < 0) continue;
    long long per = 1;
    for (int d = 0; d < plan.dim; ++d) per *= var == AFV_RHS ? plan.nc_at(l) : plan.nc_at(l) + 2;
    const long long o0 = var == AFV_RHS ? plan.offi[a] : plan.offg[a];
    const long long o1 = (var == AFV_RHS ? plan.offi[b] : plan.offg[b]) + per;
    cudaMemsetAsync(v + o0, 0, sizeof(double) * (o1 - o0), stream);
  }
  return check(err, "zero_tree");
}

int Forest::gc_tree(std::string& err) {
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) fill(d64, l, false);
  return check(err, "gc_tree");
}

// mg$D_fas_fmg, src/m_aX_mg.f90:164-203, for every tree of the forest. Trees
// of different depth finish at their own highest level: at FMG step lvl only
// trees with highest_lvl >= lvl take part.
int Forest::fmg(const MgOpts& mg, bool set_residual, bool have_guess, std::string& err) {
  const int l0 = plan.min_lvl;
  std::vector<int> all(plan.n_trees, 1);
  set_active_host(all);
  Meta m = meta_of(meta);
  if (generic()) gen_coef();
  if (have_guess) {
    for (int l = plan.max_lvl; l >= l0 + 1; --l) {
      // set_coarse_phi_rhs(l): trees with highest == l first fill level l.
      std::vector<int> top(plan.n_trees, 0);
      bool any = false;
      for (int t = 0; t < plan.n_trees; ++t)
        if (plan.tree_highest[t] == l) top[t] = 1, any = true;
      if (any) {
        set_active_host(top);
        fill(d64, l, false);
        set_active_host(all);
      }
      if (generic())
        gen_update_coarse(l, false);
      else
        update_coarse_t(d64, l, false, false);
    }
  } else if (generic()) {
    gen_init_phi_rhs();
  } else {
    // init_phi_rhs: phi = 0 on levels > min_lvl, rhs restricted downwards.
    for (int l = plan.max_lvl; l >= l0 + 1; --l) {
      int nbx = lvl_n(l);
      if (!nbx) continue;
      BoxSet bs = level_set(l);
      bool sub = l <= 1;
      with_nc(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
        constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
        using G = dev::Geo<D, NC>;
        constexpr int VW = dev::Vec<double>::w;
        long long items = (long long)nbx * (G::SG / VW);
        {
          ProfScope ps(this, kProfOther, 8.0 * nbx * G::SG);
          launch_k(dev::k_box_op<D, NC, double>, grid_for((items + 255) / 256, n_sm), 256, 0, stream, 
              m, bs, d64.phi, nullptr, 0);
        }
        constexpr int H = NC / 2;
        long long it2 = (long long)nbx * (D == 2 ? H * H : H * H * H);
        ProfScope ps(this, kProfOther, 8.0 * nbx * G::SI * (1.0 + 1.0 / (1 << D)));
        if (sub)
          launch_k(dev::k_restrict_interior<D, NC, true, double>, grid_for((it2 + 255) / 256, n_sm), 256, 0, stream, m, bs, d64.rhs);
        else
          launch_k(dev::k_restrict_interior<D, NC, false, double>, grid_for((it2 + 255) / 256, n_sm), 256, 0, stream, m, bs, d64.rhs);
      });
    }
  }
  for (int l = l0; l <= plan.max_lvl; ++l) {
    std::vector<int> act(plan.n_trees, 0);
    for (int t = 0; t < plan.n_trees; ++t) act[t] = plan.tree_highest[t] >= l;
    set_active_host(act);
    int nbx = lvl_n(l);
    if (nbx) {
      BoxSet bs = level_set(l);
      with_nc(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
        constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
        using G = dev::Geo<D, NC>;
        constexpr int VW = dev::Vec<double>::w;
        long long items = (long long)nbx * (G::SG / VW);
        ProfScope ps(this, kProfOther, 16.0 * nbx * G::SG);
        launch_k(dev::k_box_op<D, NC, double>, grid_for((items + 255) / 256, n_sm), 256, 0, stream, 
            m, bs, d64.tmp, d64.phi, 1);
      });
    }
    if (l > l0) {
      if (generic())
        gen_correct(l - 1);
      else
        correct(d64, l - 1);
      fill(d64, l, false);
    }
    if (generic())
      gen_vcycle(mg, l, false);
    else
      vcycle_t(d64, mg, l, false, false);
    if (set_residual) {
      std::vector<int> fin(plan.n_trees, 0);
      bool any = false;
      for (int t = 0; t < plan.n_trees; ++t)
        if (plan.tree_highest[t] == l) fin[t] = 1, any = true;
      if (any) {
        set_active_host(fin);
        for (int k = l0; k <= l; ++k)
          if (generic())
            gen_residual(k, nullptr);
          else
            residual(d64, k, nullptr, true);
      }
    }
  }
  set_active_host(all);
  if (int rc = check(err, "fmg")) return rc;
  return check_device_error(err);
}

int Forest::max_abs(int t, int var, double* out, std::string& err) {
  if (t < 0 || t >= plan.n_trees) return err = "tree index out of range", AFV_ERR_INVALID;
  std::vector<int> act(plan.n_trees, 0);
  act[t] = 1;
  std::vector<int> saved = host_active;
  set_active_host(act);
  norm_reset();
  Meta m = meta_of(meta);
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) {
    int nl = n_leaves(l);
    if (!nl) continue;
    BoxSet bs{leaves_list(l), 0, nl};
    const double* v = var == AFV_PHI ? d64.phi : var == AFV_RHS ? d64.rhs : d64.tmp;
    with_nc(plan.dim, plan.nc_at(l), [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
      constexpr int BPC = dev::kThreads / PER_BOX;
      ProfScope ps(this, kProfOther, 8.0 * nl * G::SI);
      launch_k(dev::k_maxabs<D, NC, double>, grid_for((nl + BPC - 1) / BPC, n_sm), dev::kThreads, 0, stream, 
          m, bs, v, var != AFV_RHS, d_norm);
    });
  }
  norm_fold();
  cudaMemcpyAsync(h_norm, d_red, sizeof(unsigned long long) * plan.n_trees, cudaMemcpyDeviceToHost,
                  stream);
  cudaStreamSynchronize(stream);
  std::memcpy(out, &h_norm[t], sizeof(double));
  set_active_host(saved);
  return check(err, "max_abs");
}

// Ghost fill of the FP64 state on all levels, coarse to fine.
void Forest::fill_all64(bool homog) {
  for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) fill(d64, l, homog);
}

// a$D_restrict_tree for phi (src/m_aX_restrict.f90:54-64), then ghost cells.
void Forest::restrict_tree_phi64() {
  for (int l = plan.max_lvl; l >= plan.min_lvl + 1; --l) restrict_res(d64, l, false);
  fill_all64(false);
}

// The fixed-point defect's shapes for the forest's leaf boxes: bit c set
// when c cells per thread (1, 2, 4) exist for them.
int Forest::defect_shapes() const {
  int bits = 0;
  with_nc(plan.dim, plan.nc, [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    if constexpr (dev::DefectFxCfg<D, NC, 1>::OK) bits |= 1;
    if constexpr (dev::DefectFxCfg<D, NC, 2>::OK) bits |= 2;
    if constexpr (dev::DefectFxCfg<D, NC, 4>::OK) bits |= 4;
  });
  return bits;
}

// Cells per thread of the fixed-point defect: the forest's choice when that
// shape exists, else the most of 4, 2, 1 that does (fewer, larger
// iterations); 0 when none does (the FP64 sum, k_defect).
int Forest::defect_cr() const {
  const int bits = defect_shapes();
  if (defect_cells > 0 && (bits & defect_cells)) return defect_cells;
  return (bits & 4) ? 4 : (bits & 2) ? 2 : (bits & 1) ? 1 : 0;
}

// The mixed solve's FP64 defect on the leaves into the FP32 right-hand side,
// with max |r| per tree into the striped norms; ghost cells are pulled inside
// the kernel.
void Forest::launch_defect() {
  Meta m = meta_of(meta);
  const int nl = n_all_leaves();
  BoxSet bs{d_lists + all_leaves_off, 0, nl};
  with_nc(plan.dim, plan.nc, [&](auto d_, auto nc_) {
    constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
    using G = dev::Geo<D, NC>;
    constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
    constexpr int BPC = dev::boxes_per_cta<G::SG, PER_BOX, double>(1);
    // read u (8 B), f (8 B); write r (4 B)
    ProfScope ps(this, kProfDefect, 20.0 * nl * G::SI);
    bool done = false;
    auto fx = [&](auto cr_) {
      constexpr int CR = decltype(cr_)::value;
      using FC = dev::DefectFxCfg<D, NC, CR>;
      if constexpr (FC::OK) {
        const int occ = kernel_occupancy((const void*)dev::k_defect_fx<D, NC, CR>, FC::T, 0);
        const long long groups = ((long long)nl + FC::LPB - 1) / FC::LPB;
        const int grid = (int)std::max(1LL, std::min(groups, (long long)n_sm * occ));
        launch_k(dev::k_defect_fx<D, NC, CR>, grid, FC::T, 0, stream, m, bs, (const double*)d64.phi,
                 (const double*)d64.rhs, d32.rhs, d_norm);
        done = true;
      }
    };
    if (defect_fx) {
      switch (defect_cr()) {
        case 1: fx(std::integral_constant<int, 1>{}); break;
        case 2: fx(std::integral_constant<int, 2>{}); break;
        case 4: fx(std::integral_constant<int, 4>{}); break;
        default: break;  // no shape for these boxes: the FP64 sum
      }
    }
    if (!done)
      launch_k(dev::k_defect<D, NC>, grid_for((nl + BPC - 1) / BPC, n_sm * 4), dev::kThreads, 0, stream, m, bs,
               d64.phi, d64.rhs, d32.rhs, d_norm);
  });
}

// One residual check, enqueued only: per-tree max |r| over the leaves (the FP64
// residual, or the FP64 defect written as the FP32 right-hand side of the
// mixed cycle), the convergence flags, each active tree's cycle count and
// last norm, and (readback) the active count copied to pinned host memory.
void Forest::enqueue_residual_check(int precision, double tol, int count_cycle) {
  const int nt = plan.n_trees;
  norm_reset();
  if (precision == AFV_PREC_MIXED) {
    launch_defect();
  } else if (generic()) {
    for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) gen_residual(l, d_norm);
  } else {
    for (int l = plan.min_lvl; l <= plan.max_lvl; ++l) residual(d64, l, d_norm, true);
  }
  cudaMemsetAsync(d_count, 0, 2 * sizeof(int), stream);
  norm_fold();
  {
    ProfScope ps(this, kProfOther, 20.0 * nt);
    launch_k(dev::k_check, (nt + 255) / 256, 256, 0, stream, nt, d_red, d_fmax, tol, meta.active, d_failed,
             d_count, (const int*)meta.err, d_cycles, d_final, count_cycle);
  }
  // the active count and the device error word, for a host-driven loop
  if (readback) cudaMemcpyAsync(h_count, d_count, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream);
}

// One solve iteration, enqueued only: a V-cycle (FP64), or an FP32 V-cycle
// on the defect with the FP64 accumulate (mixed), then the residual check.
// Work on the side stream between fork() and join() runs beside the main
// stream's (both are captured into the iteration's graph as parallel
// branches). Launch helpers take the forest's current stream, so a branch is
// enqueued with the two streams swapped.
void Forest::fork() {
  cudaEventRecord(ev_fork, stream);
  cudaStreamWaitEvent(side, ev_fork, 0);
}
void Forest::join() {
  cudaEventRecord(ev_join, side);
  cudaStreamWaitEvent(stream, ev_join, 0);
}

// One mixed iteration expects the correction array zeroed (solve() zeroes it
// before the first; each iteration zeroes it for the next beside its defect).
void Forest::enqueue_iteration(const MgOpts& mg, int precision, double tol) {
  Meta m = meta_of(meta);
  if (precision == AFV_PREC_MIXED) {
    vcycle_t(d32, mg, plan.max_lvl, true, true, true);
    int nl = n_all_leaves();
    BoxSet bs{d_lists + all_leaves_off, 0, nl};
    with_nc(plan.dim, plan.nc, [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      long long items = (long long)nl * G::SI;
      // The leaves' accumulate and the parents' increments touch disjoint
      // cells (leaves' u; parents' u and e, from the leaves' e): two branches.
      fork();
      std::swap(stream, side);
      // parents (finest first) take the restriction of their children's increments
      for (int l = plan.max_lvl - 1; l >= 1; --l) {
        int np = n_parents(l);
        if (!np) continue;
        BoxSet pb{parents_list(l), 0, np};
        long long pit = (long long)np * G::SI;
        ProfScope ps(this, kProfAccumulate, (4.0 * (1 << D) + 4.0 + 16.0) * pit);
        launch_k(dev::k_restrict_increment<D, NC>, grid_for((pit + 255) / 256, n_sm), 256, 0, stream,
                 m, pb, d64.phi, d32.phi);
      }
      std::swap(stream, side);
      {
        // read e (4 B), read and write u (16 B)
        ProfScope ps(this, kProfAccumulate, 20.0 * items);
        launch_k(dev::k_accumulate<D, NC>, grid_for((items / NC + 255) / 256, n_sm), 256, 0, stream, m, bs,
                 d64.phi, d32.phi);
      }
      join();
    });
    // the next iteration's zero correction, beside this one's defect
    fork();
    zero_correction(side);
    enqueue_residual_check(precision, tol);
    join();
  } else {
    if (generic())
      gen_vcycle(mg, plan.max_lvl, false);
    else
      vcycle_t(d64, mg, plan.max_lvl, false, false);
    enqueue_residual_check(precision, tol);
  }
}

// Set-up of a solve, enqueued only: every tree active, cycle counts zeroed,
// max |f| over each tree's leaves, parents of the mixed solve's u as the
// restriction of their children (their values are only read by coarse leaves
// next to refined regions) and the first correction zeroed, then the residual
// check before the first cycle. With a loop handle, the loop-entry decision.
void Forest::enqueue_solve_begin(int precision, double tol, int max_cycles, const cudaGraphConditionalHandle* h) {
  const int nt = plan.n_trees;
  Meta m = meta_of(meta);
  // the trees this solve takes part in
  cudaMemcpyAsync(meta.active, d_solve_mask, sizeof(int) * nt, cudaMemcpyDeviceToDevice, stream);
  cudaMemsetAsync(d_cycles, 0, sizeof(int) * nt, stream);
  cudaMemsetAsync(d_failed, 0, sizeof(int) * nt, stream);
  if (generic()) gen_coef();
  norm_reset();
  {
    // all leaves are on levels >= 1, with nc cells per side: one launch
    const int nl = n_all_leaves();
    BoxSet bs{d_lists + all_leaves_off, 0, nl};
    with_nc(plan.dim, plan.nc, [&](auto d_, auto nc_) {
      constexpr int D = decltype(d_)::value, NC = decltype(nc_)::value;
      using G = dev::Geo<D, NC>;
      constexpr int PER_BOX = G::SI < dev::kThreads ? G::SI : dev::kThreads;
      constexpr int BPC = dev::kThreads / PER_BOX;
      ProfScope ps(this, kProfOther, 8.0 * nl * G::SI);
      launch_k(dev::k_maxabs<D, NC, double>, grid_for((nl + BPC - 1) / BPC, n_sm * 4), dev::kThreads, 0,
               stream, m, bs, d64.rhs, 0, d_norm);
    });
  }
  norm_fold();
  cudaMemcpyAsync(d_fmax, d_red, sizeof(double) * nt, cudaMemcpyDeviceToDevice, stream);
  if (precision == AFV_PREC_MIXED) {
    for (int l = plan.max_lvl; l >= plan.min_lvl + 1; --l) restrict_res(d64, l, false);
    zero_correction(stream);  // the first correction
  }
  enqueue_residual_check(precision, tol, 0);
  if (h) {
    dev::k_loop_start<<<1, 1, 0, stream>>>(*h, d_count, max_cycles);
    ++n_launches;
  }
}

// Finish of a solve, enqueued only: the mixed solve's state completed
// (parents as restrictions, ghost cells filled), every tree active again, and
// the results copied to pinned host memory.
void Forest::enqueue_solve_end(int precision) {
  const int nt = plan.n_trees;
  if (precision == AFV_PREC_MIXED) {
    // the parents of u and the ghost cells of the trees this solve took part
    // in (the others stay as they were)
    cudaMemcpyAsync(meta.active, d_solve_mask, sizeof(int) * nt, cudaMemcpyDeviceToDevice, stream);
    restrict_tree_phi64();
  }
  dev::k_set_int<<<(nt + 255) / 256, 256, 0, stream>>>(meta.active, nt, 1);
  ++n_launches;
  cudaMemcpyAsync(h_count, d_count, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(h_cycles, d_cycles, sizeof(int) * nt, cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(h_final, d_final, sizeof(unsigned long long) * nt, cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(h_failed, d_failed, sizeof(int) * nt, cudaMemcpyDeviceToHost, stream);
  cudaMemcpyAsync(h_fmax, d_fmax, sizeof(double) * nt, cudaMemcpyDeviceToHost, stream);
}

// Captures a whole solve into one graph: the set-up, a conditional while node
// whose body is one iteration followed by k_loop_step (captured on
// loop_stream, with side for its parallel branches), and the finish. The
// device decides every repetition, so a solve is one launch and one host
// synchronisation.
int Forest::build_solve_graph(GraphCache& gc, const MgOpts& mg, int precision, double tol, int max_cycles,
                              std::string& err) {
  if (gc.exec) cudaGraphExecDestroy(gc.exec);
  gc = GraphCache();
  std::lock_guard<std::mutex> lock(g_capture_mutex);
  cudaGraph_t top = nullptr;
  cudaGraphConditionalHandle h = 0;
  cudaGraphNode_t loop = nullptr;
  cudaGraph_t body = nullptr;
  readback = false;
  const long long n0 = n_launches;
  bool ok = cudaGraphCreate(&top, 0) == cudaSuccess &&
            cudaGraphConditionalHandleCreate(&h, top, 0, cudaGraphCondAssignDefault) == cudaSuccess &&
            cudaStreamBeginCaptureToGraph(stream, top, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) ==
                cudaSuccess;
  if (ok) {
    enqueue_solve_begin(precision, tol, max_cycles, &h);
    gc.k_pre = n_launches - n0;
    // the loop node after what has been captured so far
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    ok = cudaStreamGetCaptureInfo(stream, &cs, nullptr, &cg, &deps, &edges, &nd) == cudaSuccess &&
         cs == cudaStreamCaptureStatusActive;
    if (ok) {
      cudaGraphNodeParams np = {};
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      ok = cudaGraphAddNode(&loop, cg, deps, nullptr, nd, &np) == cudaSuccess &&
           cudaStreamUpdateCaptureDependencies(stream, &loop, nullptr, 1, cudaStreamSetCaptureDependencies) ==
               cudaSuccess;
      if (ok) body = np.conditional.phGraph_out[0];
    }
    if (ok) {
      std::swap(stream, loop_stream);
      ok = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) ==
           cudaSuccess;
      if (ok) {
        const long long n1 = n_launches;
        enqueue_iteration(mg, precision, tol);
        dev::k_loop_step<<<1, 1, 0, stream>>>(h, d_count, max_cycles);
        ++n_launches;
        gc.k_body = n_launches - n1;
        cudaGraph_t b = nullptr;
        ok = cudaStreamEndCapture(stream, &b) == cudaSuccess;
      }
      std::swap(stream, loop_stream);
    }
    const long long n2 = n_launches;
    enqueue_solve_end(precision);
    gc.k_post = n_launches - n2;
    cudaGraph_t t = nullptr;
    const bool ended = cudaStreamEndCapture(stream, &t) == cudaSuccess;
    ok = ok && ended;
  }
  n_launches = n0;
  readback = true;
  if (ok) ok = cudaGraphInstantiate(&gc.exec, top, 0) == cudaSuccess;
  if (top) cudaGraphDestroy(top);
  if (!ok) {
    if (gc.exec) cudaGraphExecDestroy(gc.exec);
    gc = GraphCache();
    if (int rc = check(err, "solve graph")) return rc;
    return err = "solve graph: capture failed", AFV_ERR_CUDA;
  }
  gc.n_down = mg.n_down;
  gc.n_up = mg.n_up;
  gc.n_base = mg.n_base;
  gc.tol = tol;
  gc.max_cycles = max_cycles;
  return AFV_OK;
}

// Solve every tree to max|f - L phi| <= tol * max|f| over its leaves. With
// graphs on (and the profiler off) the whole solve is one CUDA-graph launch,
// captured on first use: the iterations repeat on the device (a conditional
// while node) until no tree is active, max_cycles is reached or a bounded
// wait gave up. Trees that have converged are masked out on the device, so the
// graph does not change while the set of active trees shrinks. Otherwise the
// host drives the loop, one iteration at a time.
int Forest::solve(const MgOpts& mg, int precision, double tol, int max_cycles, SolveStats& st,
                  std::string& err, const int* mask) {
  const int nt = plan.n_trees;
  // A mask of leading trees (a forest whose first k slots hold requests):
  // the launches cover those trees' boxes only (tree_limit).
  int lead = 0;
  bool prefix = mask != nullptr;
  if (mask) {
    while (lead < nt && mask[lead]) ++lead;
    for (int t = lead; t < nt; ++t)
      if (mask[t]) prefix = false;
  }
  struct LimitScope {
    Forest* f;
    ~LimitScope() { f->tree_limit = 0; }
  } limit_scope{this};
  tree_limit = (prefix && lead > 0 && lead < nt) ? lead : 0;
  for (int t = 0; t < nt; ++t) h_solve_mask[t] = mask ? (mask[t] != 0) : 1;
  cudaMemcpyAsync(d_solve_mask, h_solve_mask, sizeof(int) * nt, cudaMemcpyHostToDevice, stream);
  if (precision == AFV_PREC_MIXED && !mixed)
    return err = "forest created without mixed_buffers", AFV_ERR_STATE;
  if (precision == AFV_PREC_MIXED && generic())
    return err = "mixed-precision solves take the Cartesian constant-coefficient operator only", AFV_ERR_UNSUPPORTED;
  st.cycles.assign(nt, 0);
  st.rel_res.assign(nt, 0.0);
  const bool graph = use_graphs && prof_mask == 0;
  if (graph) {
    GraphCache& gc = graph_for(precision, tree_limit);
    if (!gc.exec || gc.n_down != mg.n_down || gc.n_up != mg.n_up || gc.n_base != mg.n_base || gc.tol != tol ||
        gc.max_cycles != max_cycles)
      if (int rc = build_solve_graph(gc, mg, precision, tol, max_cycles, err)) return rc;
    if (cudaGraphLaunch(gc.exec, stream) != cudaSuccess) return check(err, "graph launch");
    if (cudaStreamSynchronize(stream) != cudaSuccess) return check(err, "solve");
    n_launches += gc.k_pre + gc.k_post + gc.k_body * h_count[2];
  } else {
    enqueue_solve_begin(precision, tol, max_cycles, nullptr);
    if (cudaStreamSynchronize(stream) != cudaSuccess) return check(err, "solve");
    int cyc = 0;
    while (h_count[0] > 0 && cyc < max_cycles && !h_count[1]) {
      if (prof_mask && prof_lead_us > 0) dev::k_hold<<<1, 1, 0, stream>>>(1000LL * prof_lead_us);
      enqueue_iteration(mg, precision, tol);
      if (cudaStreamSynchronize(stream) != cudaSuccess) return check(err, "solve");
      ++cyc;
      if (int rc = check(err, "solve")) return rc;
    }
    enqueue_solve_end(precision);
    if (cudaStreamSynchronize(stream) != cudaSuccess) return check(err, "solve");
  }
  host_active.assign(nt, 1);
  if (int rc = check(err, "solve")) return rc;
  if (h_count[1]) return check_device_error(err);  // a bounded wait gave up
  int n_failed = 0;
  for (int t = 0; t < nt; ++t) {
    if (!h_solve_mask[t]) continue;  // left out of this solve
    double r;
    std::memcpy(&r, &h_final[t], sizeof(double));
    st.cycles[t] = h_cycles[t];
    st.rel_res[t] = h_fmax[t] > 0 ? r / h_fmax[t] : r;
    n_failed += h_failed[t] != 0;
  }
  const int n_active = h_count[0];
  st.status = n_failed ? AFV_ERR_DIVERGED : n_active > 0 ? AFV_ERR_NOT_CONVERGED : AFV_OK;
  if (n_failed)
    err = std::to_string(n_failed) + " tree(s) diverged (non-finite residual)";
  else if (n_active > 0)
    err = "not converged within max_cycles";
  return st.status;
}

}  // namespace afv

#include "noalloc.cuh"  // Forest::max_abs_static
