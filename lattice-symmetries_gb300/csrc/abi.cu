// abi.cu -- C ABI of libls_gb300.so: the drop-in ls_hs_* / ls_chpl_* symbols and the additive
// ls_gpu_* symbols declared in include/ls_gb300.h.  Host logic only; kernels live in basis.cu
// and matvec*.cu.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <unistd.h>

#include "lsg.h"

namespace lsg {
int set_matvec_config(int threads, int blocks_per_sm);
int set_matvec_rhs_tile(int tile);
void get_matvec_config(int* threads, int* waves, int* rhs_tile);
int set_block_arithmetic(int mode);
int get_block_arithmetic();
}

using namespace lsg;

// =================================================================================================
// Runtime state
// =================================================================================================
namespace {

std::mutex g_mutex;  // serialises the host-pointer entry points (the reference is not re-entrant
                     // either: reference.c:213 "not thread-safe")
thread_local std::string g_last_error;

struct Scratch {
  void* ptr = nullptr;
  size_t size = 0;
};
struct DeviceRuntime {
  bool ready = false;
  cudaStream_t stream = nullptr;
  int sms = 0;
  int* err_word = nullptr;        // device
  uint64_t* binom = nullptr;      // device 65x65
  Scratch dev[12];
  Scratch host[12];
};
DeviceRuntime g_rt[16];

int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return (d >= 0 && d < 16) ? d : 0;
}

DeviceRuntime& rt() {
  DeviceRuntime& r = g_rt[current_device()];
  if (!r.ready) {
    cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking);
    int dev = current_device();
    cudaDeviceGetAttribute(&r.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaMalloc((void**)&r.err_word, 4 * sizeof(int));
    cudaMemset(r.err_word, 0, 4 * sizeof(int));
    uint64_t table[65][65];
    memset(table, 0, sizeof(table));
    table[0][0] = 1;
    for (int n = 1; n <= 64; ++n) {
      table[n][0] = 1;
      for (int k = 1; k <= n; ++k) table[n][k] = table[n - 1][k - 1] + table[n - 1][k];
    }
    cudaMalloc((void**)&r.binom, sizeof(table));
    cudaMemcpy(r.binom, table, sizeof(table), cudaMemcpyHostToDevice);
    // Stream-ordered allocations (the matvec's prescaled gather source, scan scratch) come from
    // the device's default memory pool: keep freed blocks in this process's pool instead of
    // returning them at every synchronisation, so that repeated matvecs (and graph replays) do
    // not map memory again.  A process-local allocator attribute, not a device setting.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    r.ready = true;
  }
  return r;
}

// default handler: print and abort, like reference.c:20-23
void default_error_handler(char const* message) {
  fprintf(stderr, "[Error]   %s\n[Error]   Aborting ...", message);
  abort();
}
std::atomic<void (*)(char const*)> g_handler{&default_error_handler};

}  // namespace

namespace lsg {

cudaStream_t default_stream() { return rt().stream; }
int num_sms() { return std::max(1, rt().sms); }
void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}
int* device_error_word() { return rt().err_word; }
const uint64_t* device_binomials() { return rt().binom; }

void* scratch(size_t bytes, int slot) {
  Scratch& s = rt().dev[slot];
  if (s.size < bytes) {
    if (s.ptr) cudaFree(s.ptr);
    s.ptr = nullptr;
    s.size = 0;
    size_t want = std::max<size_t>(bytes, 1 << 20);
    if (cudaMalloc(&s.ptr, want) != cudaSuccess) {
      s.ptr = nullptr;
      g_last_error = "out of device memory for a scratch buffer";
      return nullptr;
    }
    s.size = want;
  }
  return s.ptr;
}

void* pinned_scratch(size_t bytes, int slot) {
  Scratch& s = rt().host[slot];
  if (s.size < bytes) {
    if (s.ptr) cudaFreeHost(s.ptr);
    s.ptr = nullptr;
    s.size = 0;
    size_t want = std::max<size_t>(bytes, 1 << 20);
    if (cudaMallocHost(&s.ptr, want) != cudaSuccess) {
      s.ptr = nullptr;
      g_last_error = "out of pinned host memory for a staging buffer";
      return nullptr;
    }
    s.size = want;
  }
  return s.ptr;
}

}  // namespace lsg

// =================================================================================================
// Error handling (reference.c:11-36)
// =================================================================================================
extern "C" void ls_hs_fatal_error(char const* func, int line, char const* message) {
  fprintf(stderr, "[Error]   [%s#%i] %s\n[Error]   Aborting ...", func, line, message);
  abort();
}

extern "C" void ls_hs_set_exception_handler(void (*handler)(char const* message)) {
  g_handler.store(handler == nullptr ? &default_error_handler : handler);
}

extern "C" void ls_hs_error(char const* message) {
  auto h = g_handler.load();
  if (h == nullptr) ls_hs_fatal_error(__func__, __LINE__, "error handler is NULL");
  h(message);
}

static void report(const char* prefix) {
  std::string m = std::string(prefix) + (g_last_error.empty() ? "" : (": " + g_last_error));
  ls_hs_error(m.c_str());
}

extern "C" char const* ls_gpu_last_error(void) { return g_last_error.c_str(); }

// =================================================================================================
// External arrays and refcounts (reference.c:38-64)
// =================================================================================================
extern "C" void ls_hs_internal_destroy_external_array(chpl_external_array* arr) {
  if (arr == nullptr) ls_hs_fatal_error(__func__, __LINE__, "trying to destroy a NULL chpl_external_array");
  if (arr->freer != nullptr) {
    auto f = (void (*)(void*))arr->freer;
    f(arr->elts);
  }
}
extern "C" int ls_hs_internal_read_refcount(ls_gb300_refcount const* rc) {
  return __atomic_load_n(rc, __ATOMIC_SEQ_CST);
}
extern "C" void ls_hs_internal_write_refcount(ls_gb300_refcount* rc, int value) {
  __atomic_store_n(rc, value, __ATOMIC_SEQ_CST);
}
extern "C" int ls_hs_internal_inc_refcount(ls_gb300_refcount* rc) {
  return __atomic_fetch_add(rc, 1, __ATOMIC_SEQ_CST);
}
extern "C" int ls_hs_internal_dec_refcount(ls_gb300_refcount* rc) {
  return __atomic_fetch_sub(rc, 1, __ATOMIC_SEQ_CST);
}

static void free_pinned(void* p) {
  if (p) cudaFreeHost(p);
}
static void free_malloced(void* p) { free(p); }

// =================================================================================================
// Plugin table (reference.c:213-225) and library start-up
// =================================================================================================
static ls_chpl_kernels g_chpl_kernels = {nullptr, nullptr, nullptr, nullptr};

extern "C" ls_chpl_kernels const* ls_hs_internal_get_chpl_kernels(void) { return &g_chpl_kernels; }
extern "C" void ls_hs_internal_set_chpl_kernels(ls_chpl_kernels const* kernels) {
  g_chpl_kernels = *kernels;
}

static void install_gpu_drivers() {
  ls_chpl_kernels k;
  k.enumerate_states = (void (*)(ls_hs_basis const*, uint64_t, uint64_t, chpl_external_array*))
      & ls_chpl_enumerate_representatives;
  k.operator_apply_off_diag = &ls_chpl_operator_apply_off_diag;
  k.operator_apply_diag = &ls_chpl_operator_apply_diag;
  k.matrix_vector_product = &ls_chpl_matrix_vector_product;
  ls_hs_internal_set_chpl_kernels(&k);
}

// The reference's Chapel library installs its drivers when its module initialises
// (LatticeSymmetries.chpl:17-32); this library does the same when it is loaded.
__attribute__((constructor)) static void lsg_on_load() { install_gpu_drivers(); }

extern "C" void ls_chpl_init(void) { install_gpu_drivers(); }
extern "C" void ls_chpl_init_kernels(void) { install_gpu_drivers(); }
extern "C" void chpl__init_LatticeSymmetries(int64_t, int32_t) { install_gpu_drivers(); }
extern "C" void chpl__init_BatchedOperator(int64_t, int32_t) {}
extern "C" void chpl__init_CommonParameters(int64_t, int32_t) {}
extern "C" void chpl__init_ConcurrentAccessor(int64_t, int32_t) {}
extern "C" void chpl__init_DistributedMatrixVector(int64_t, int32_t) {}
extern "C" void chpl__init_FFI(int64_t, int32_t) {}
extern "C" void chpl__init_ForeignTypes(int64_t, int32_t) {}
extern "C" void chpl__init_StatesEnumeration(int64_t, int32_t) {}
extern "C" void chpl__init_Vector(int64_t, int32_t) {}
extern "C" void ls_chpl_finalize(void) {
  std::lock_guard<std::mutex> lock(g_mutex);
  for (int d = 0; d < 16; ++d) {
    DeviceRuntime& r = g_rt[d];
    if (!r.ready) continue;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(d);
    for (auto& s : r.dev) {
      if (s.ptr) cudaFree(s.ptr);
      s = Scratch{};
    }
    for (auto& s : r.host) {
      if (s.ptr) cudaFreeHost(s.ptr);
      s = Scratch{};
    }
    cudaSetDevice(prev);
  }
}

extern "C" int ls_gpu_device_synchronize(void) {
  return cuda_ok(cudaStreamSynchronize(default_stream()), "synchronize") ? 0 : LS_GPU_ERR_CUDA;
}

extern "C" int ls_gpu_set_matvec_rhs_tile(int rhs_tile) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const int rc = set_matvec_rhs_tile(rhs_tile);
  return rc != 0 ? fail(rc, "the right-hand-side tile must be 1, 4, 8 or 16") : 0;
}

extern "C" int ls_gpu_set_block_arithmetic(int mode) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (set_block_arithmetic(mode) != 0)
    return fail(LS_GPU_ERR_INVALID, "block arithmetic: 0 = FP64, 1 = FP32 pairs for small groups, 2 = FP32 pairs");
  return 0;
}

extern "C" int ls_gpu_get_block_arithmetic(void) {
  std::lock_guard<std::mutex> lock(g_mutex);
  return get_block_arithmetic();
}

extern "C" int ls_gpu_get_matvec_config(int* threads_per_block, int* waves, int* rhs_tile) {
  std::lock_guard<std::mutex> lock(g_mutex);
  get_matvec_config(threads_per_block, waves, rhs_tile);
  return 0;
}

extern "C" int ls_gpu_set_matvec_config(int threads_per_block, int blocks_per_sm) {
  if (threads_per_block != 0 && (threads_per_block % 32 != 0 || threads_per_block > 320))
    return fail(LS_GPU_ERR_INVALID, "threads_per_block must be a multiple of 32, at most 320");
  if (blocks_per_sm < 0 || blocks_per_sm > 64) return fail(LS_GPU_ERR_INVALID, "waves must be in [0, 64]");
  return set_matvec_config(threads_per_block, blocks_per_sm);
}

// =================================================================================================
// Orbit-scan kernel data (kernels.c:112-193)
// =================================================================================================
static void* create_orbit_data(ls_hs_permutation_group const* g, int spin_inversion, int fermionic_sites);

extern "C" void* ls_internal_create_halide_kernel_data(ls_hs_permutation_group const* g,
                                                       int spin_inversion) {
  return create_orbit_data(g, spin_inversion, 0);
}

// Orbit data of a lattice-symmetry group acting on spinful fermions: `g` permutes the 2n orbitals
// (up k -> k, down k -> n + k) and carries the characters; every element acts with the sign of
// the permutation it induces on the occupied orbitals.  No counterpart in the reference, whose
// fermionic bases have no lattice symmetries (Basis.hs:713-723).
extern "C" void* ls_gpu_create_fermionic_kernel_data(ls_hs_permutation_group const* g, int number_sites) {
  if (g == nullptr || number_sites <= 0 || g->number_bits != 2 * number_sites) {
    std::lock_guard<std::mutex> lock(g_mutex);
    set_error("a fermionic group acts on 2 * number_sites orbitals");
    report("ls_gpu_create_fermionic_kernel_data");
    return nullptr;
  }
  return create_orbit_data(g, 0, number_sites);
}

static void* create_orbit_data(ls_hs_permutation_group const* g, int spin_inversion, int fermionic_sites) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (g == nullptr) {
    set_error("permutation group is NULL");
    report("ls_internal_create_halide_kernel_data");
    return nullptr;
  }
  if (spin_inversion != 0 && spin_inversion != 1 && spin_inversion != -1)
    ls_hs_fatal_error(__func__, __LINE__, "invalid spin_inversion");
  if (g->number_bits < 0 || g->number_bits > 64 || g->number_masks < 0 ||
      g->number_masks > kMaxGroupElements || g->number_shifts < 0 || g->number_shifts > 64) {
    set_error("unsupported permutation group (bits <= 64, |G| <= 2048)");
    report("ls_internal_create_halide_kernel_data");
    return nullptr;
  }
  OrbitData* od = new OrbitData();
  od->magic = kOrbitMagic;
  od->n_bits = g->number_bits;
  od->n_elems = g->number_masks;
  od->depth = g->number_shifts;
  od->spin_inversion = spin_inversion;
  const size_t nm = (size_t)od->depth * od->n_elems;
  od->masks.assign(g->masks, g->masks + nm);
  od->shifts.resize(od->depth);
  for (int k = 0; k < od->depth; ++k) od->shifts[k] = (uint32_t)g->shifts[k];
  od->chars_re.assign(g->eigvals_re, g->eigvals_re + od->n_elems);
  od->chars_im.assign(g->eigvals_im, g->eigvals_im + od->n_elems);
  od->fermionic = fermionic_sites > 0 ? 1 : 0;
  if (compute_site_images(od) != 0) {
    report("ls_internal_create_halide_kernel_data");
    delete od;
    return nullptr;
  }
  return od;
}

extern "C" void ls_internal_destroy_halide_kernel_data(void* p) {
  if (p == nullptr) return;
  OrbitData* od = (OrbitData*)p;
  if (od->magic != kOrbitMagic) return;
  if (od->dev_block) cudaFree(od->dev_block);
  od->magic = 0;
  delete od;
}

// Host-pointer staging helpers ------------------------------------------------------------------
static const uint64_t* stage_alphas(ptrdiff_t n, uint64_t const* alphas, ptrdiff_t stride, int slot) {
  uint64_t* h = (uint64_t*)pinned_scratch((size_t)n * 8, slot);
  uint64_t* d = (uint64_t*)scratch((size_t)n * 8, slot);
  if (!h || !d) return nullptr;
  if (stride == 1) {
    memcpy(h, alphas, (size_t)n * 8);
  } else {
    for (ptrdiff_t i = 0; i < n; ++i) h[i] = alphas[i * stride];
  }
  if (!cuda_ok(cudaMemcpyAsync(d, h, (size_t)n * 8, cudaMemcpyHostToDevice, default_stream()), "H2D"))
    return nullptr;
  return d;
}

extern "C" void ls_hs_state_info_halide_kernel(ptrdiff_t batch_size, uint64_t const* alphas,
                                               ptrdiff_t alphas_stride, uint64_t* betas,
                                               ptrdiff_t betas_stride, ls_hs_scalar* characters,
                                               double* norms, void const* private_data) {
  if (batch_size <= 0) return;
  std::lock_guard<std::mutex> lock(g_mutex);
  const OrbitData* od = (const OrbitData*)private_data;
  if (od == nullptr || od->magic != kOrbitMagic) {
    set_error("invalid kernel data");
    report("ls_hs_state_info");
    return;
  }
  cudaStream_t s = default_stream();
  const uint64_t* d_x = stage_alphas(batch_size, alphas, alphas_stride, 0);
  uint64_t* d_r = (uint64_t*)scratch((size_t)batch_size * 8, 1);
  double2* d_c = (double2*)scratch((size_t)batch_size * 16, 2);
  double* d_n = (double*)scratch((size_t)batch_size * 8, 3);
  uint8_t* h = (uint8_t*)pinned_scratch((size_t)batch_size * 32, 1);
  if (!d_x || !d_r || !d_c || !d_n || !h) {
    report("ls_hs_state_info");
    return;
  }
  const DeviceGroup* dg = od->n_elems > 0 ? orbit_device(od) : nullptr;
  int rc = dg ? launch_state_info(*dg, batch_size, d_x, d_r, d_c, d_n, 8, s) : LS_GPU_ERR_CUDA;
  if (od->n_elems == 0) {
    set_error("state_info requires a non-empty symmetry group");
    rc = LS_GPU_ERR_INVALID;
  }
  uint64_t* hr = (uint64_t*)h;
  double2* hc = (double2*)(h + (size_t)batch_size * 8);
  double* hn = (double*)(h + (size_t)batch_size * 24);
  if (rc == 0 &&
      (!cuda_ok(cudaMemcpyAsync(hr, d_r, (size_t)batch_size * 8, cudaMemcpyDeviceToHost, s), "D2H") ||
       !cuda_ok(cudaMemcpyAsync(hc, d_c, (size_t)batch_size * 16, cudaMemcpyDeviceToHost, s), "D2H") ||
       !cuda_ok(cudaMemcpyAsync(hn, d_n, (size_t)batch_size * 8, cudaMemcpyDeviceToHost, s), "D2H") ||
       !cuda_ok(cudaStreamSynchronize(s), "state_info")))
    rc = LS_GPU_ERR_CUDA;
  if (rc != 0) {
    report("ls_hs_state_info");
    return;
  }
  double* cout = reinterpret_cast<double*>(characters);
  for (ptrdiff_t i = 0; i < batch_size; ++i) {
    betas[i * betas_stride] = hr[i];
    cout[2 * i] = hc[i].x;
    cout[2 * i + 1] = hc[i].y;
    norms[i] = hn[i];
  }
}

extern "C" void ls_hs_is_representative_halide_kernel(ptrdiff_t batch_size, uint64_t const* alphas,
                                                      ptrdiff_t alphas_stride,
                                                      uint8_t* are_representatives, double* norms,
                                                      void const* private_data) {
  if (batch_size <= 0) return;
  std::lock_guard<std::mutex> lock(g_mutex);
  const OrbitData* od = (const OrbitData*)private_data;
  if (od == nullptr || od->magic != kOrbitMagic || od->n_elems == 0) {
    set_error("invalid kernel data or empty group");
    report("ls_hs_is_representative");
    return;
  }
  cudaStream_t s = default_stream();
  const uint64_t* d_x = stage_alphas(batch_size, alphas, alphas_stride, 0);
  uint8_t* d_f = (uint8_t*)scratch((size_t)batch_size, 1);
  double* d_n = (double*)scratch((size_t)batch_size * 8, 2);
  uint8_t* h = (uint8_t*)pinned_scratch((size_t)batch_size * 16, 1);
  if (!d_x || !d_f || !d_n || !h) {
    report("ls_hs_is_representative");
    return;
  }
  const DeviceGroup* dg = orbit_device(od);
  int rc = dg ? launch_is_representative(*dg, batch_size, d_x, d_f, d_n, 4, s) : LS_GPU_ERR_CUDA;
  double* hn = (double*)h;
  uint8_t* hf = h + (size_t)batch_size * 8;
  if (rc == 0 &&
      (!cuda_ok(cudaMemcpyAsync(hn, d_n, (size_t)batch_size * 8, cudaMemcpyDeviceToHost, s), "D2H") ||
       !cuda_ok(cudaMemcpyAsync(hf, d_f, (size_t)batch_size, cudaMemcpyDeviceToHost, s), "D2H") ||
       !cuda_ok(cudaStreamSynchronize(s), "is_representative")))
    rc = LS_GPU_ERR_CUDA;
  if (rc != 0) {
    report("ls_hs_is_representative");
    return;
  }
  memcpy(are_representatives, hf, (size_t)batch_size);
  memcpy(norms, hn, (size_t)batch_size * 8);
}

// =================================================================================================
// State index (indexing.c:94-125, :273-325)
// =================================================================================================
namespace {
// Device copies of representatives produced by the GPU enumeration, keyed by the host array they
// were copied to, so that building the index does not upload them again.
std::unordered_map<const void*, uint64_t*> g_pending_device_reps;
}

struct ls_hs_state_index_binary_search_data : IndexData {};

extern "C" ls_hs_state_index_binary_search_data* ls_hs_create_state_index_binary_search_kernel_data(
    chpl_external_array const* representatives, int number_bits, int prefix_bits) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (representatives == nullptr) ls_hs_fatal_error(__func__, __LINE__, "representatives is NULL");
  if (!(0 < number_bits && number_bits <= 64))
    ls_hs_fatal_error(__func__, __LINE__, "invalid bits");
  auto* ix = new ls_hs_state_index_binary_search_data();
  ix->magic = kIndexMagic;
  ix->n_states = (int64_t)representatives->num_elts;
  ix->host_reps = (const uint64_t*)representatives->elts;
  ix->number_bits = number_bits;
  ix->prefix_bits = std::min(prefix_bits, number_bits);
  cudaStream_t s = default_stream();
  auto it = g_pending_device_reps.find(representatives->elts);
  if (it != g_pending_device_reps.end()) {
    ix->d_reps = it->second;
    g_pending_device_reps.erase(it);
  } else {
    if (!cuda_ok(cudaMalloc((void**)&ix->d_reps, std::max<int64_t>(ix->n_states, 1) * 8), "cudaMalloc(reps)") ||
        (ix->n_states > 0 &&
         !cuda_ok(cudaMemcpyAsync(ix->d_reps, ix->host_reps, (size_t)ix->n_states * 8,
                                  cudaMemcpyHostToDevice, s), "upload reps"))) {
      report("ls_hs_create_state_index_binary_search_kernel_data");
      delete ix;
      return nullptr;
    }
  }
  int shift = 0;
  int64_t range = 0;
  uint64_t max_state = 0;
  if (build_prefix_index(ix->d_reps, ix->n_states, number_bits, ix->prefix_bits, &ix->d_offsets,
                         &range, &shift, s, &max_state, &ix->d_suffix) != 0 ||
      !cuda_ok(cudaStreamSynchronize(s), "build index")) {
    report("ls_hs_create_state_index_binary_search_kernel_data");
    cudaFree(ix->d_reps);
    delete ix;
    return nullptr;
  }
  ix->dev.n_states = ix->n_states;
  ix->dev.reps = ix->d_reps;
  ix->dev.offsets = ix->d_offsets;
  ix->dev.suffix16 = ix->d_suffix;
  ix->dev.shift = shift;
  ix->dev.range_size = range;
  ix->dev.prefix_bits = ix->prefix_bits;
  ix->dev.max_state = max_state;
  return ix;
}

extern "C" void ls_hs_destroy_state_index_binary_search_kernel_data(
    ls_hs_state_index_binary_search_data* cache) {
  if (cache == nullptr || cache->magic != kIndexMagic) return;
  cudaFree(cache->d_reps);
  cudaFree(cache->d_offsets);
  cudaFree(cache->d_suffix);
  cudaFree(cache->d_norms);
  cache->magic = 0;
  delete cache;
}

extern "C" void ls_hs_state_index_binary_search_kernel(ptrdiff_t batch_size, uint64_t const* spins,
                                                       ptrdiff_t spins_stride, ptrdiff_t* indices,
                                                       ptrdiff_t indices_stride,
                                                       void const* private_kernel_data) {
  if (indices_stride != 1) ls_hs_fatal_error(__func__, __LINE__, "expected indices_stride==1");
  if (spins_stride != 1) ls_hs_fatal_error(__func__, __LINE__, "expected spins_stride==1");
  if (batch_size <= 0) return;
  std::lock_guard<std::mutex> lock(g_mutex);
  const IndexData* ix = (const IndexData*)private_kernel_data;
  if (ix == nullptr || ix->magic != kIndexMagic) {
    set_error("invalid index data");
    report("ls_hs_state_index");
    return;
  }
  cudaStream_t s = default_stream();
  const uint64_t* d_x = stage_alphas(batch_size, spins, 1, 0);
  int64_t* d_i = (int64_t*)scratch((size_t)batch_size * 8, 1);
  if (!d_x || !d_i) {
    report("ls_hs_state_index");
    return;
  }
  int rc = launch_state_index(ix->dev, batch_size, d_x, d_i, s);
  if (rc == 0 && (!cuda_ok(cudaMemcpyAsync(indices, d_i, (size_t)batch_size * 8, cudaMemcpyDeviceToHost, s), "D2H") ||
                  !cuda_ok(cudaStreamSynchronize(s), "state_index")))
    rc = LS_GPU_ERR_CUDA;
  if (rc != 0) report("ls_hs_state_index");
}

// =================================================================================================
// Dispatchers (reference.c:137-171)
// =================================================================================================
extern "C" void ls_hs_state_index(ls_hs_basis const* basis, ptrdiff_t batch_size, uint64_t const* spins,
                                  ptrdiff_t spins_stride, ptrdiff_t* indices, ptrdiff_t indices_stride) {
  if (basis->kernels->state_index_kernel == nullptr)
    ls_hs_fatal_error(__func__, __LINE__, "state_index_kernel is NULL");
  basis->kernels->state_index_kernel(batch_size, spins, spins_stride, indices, indices_stride,
                                     basis->kernels->state_index_data);
}

extern "C" void ls_hs_is_representative(ls_hs_basis const* basis, ptrdiff_t batch_size,
                                        uint64_t const* alphas, ptrdiff_t alphas_stride,
                                        uint8_t* are_representatives, double* norms) {
  if (basis->kernels->is_representative_kernel == nullptr)
    ls_hs_fatal_error(__func__, __LINE__,
                      "is_representative_kernel is NULL, perhaps this basis requires no projection?");
  basis->kernels->is_representative_kernel(batch_size, alphas, alphas_stride, are_representatives,
                                           norms, basis->kernels->is_representative_data);
}

extern "C" void ls_hs_state_info(ls_hs_basis const* basis, ptrdiff_t batch_size, uint64_t const* alphas,
                                 ptrdiff_t alphas_stride, uint64_t* betas, ptrdiff_t betas_stride,
                                 ls_hs_scalar* characters, double* norms) {
  if (basis->kernels->state_info_kernel == nullptr)
    ls_hs_fatal_error(__func__, __LINE__,
                      "state_info_kernel is NULL, perhaps this basis requires no projection?");
  basis->kernels->state_info_kernel(batch_size, alphas, alphas_stride, betas, betas_stride,
                                    characters, norms, basis->kernels->state_info_data);
}

// =================================================================================================
// Basis helpers
// =================================================================================================
static int basis_number_bits(ls_hs_basis const* b) {
  return (b->particle_type == LS_HS_SPINFUL_FERMION ? 2 : 1) * b->number_sites;
}

static const OrbitData* basis_orbit(ls_hs_basis const* b) {
  if (b->kernels == nullptr) return nullptr;
  if (b->kernels->state_info_kernel != &ls_hs_state_info_halide_kernel) return nullptr;
  const OrbitData* od = (const OrbitData*)b->kernels->state_info_data;
  return (od && od->magic == kOrbitMagic) ? od : nullptr;
}

static IndexData* basis_index(ls_hs_basis const* b) {
  if (b->kernels == nullptr) return nullptr;
  if (b->kernels->state_index_kernel != &ls_hs_state_index_binary_search_kernel) return nullptr;
  IndexData* ix = (IndexData*)b->kernels->state_index_data;
  return (ix && ix->magic == kIndexMagic) ? ix : nullptr;
}

static bool has_permutations(ls_hs_basis const* b) {
  const OrbitData* od = basis_orbit(b);
  if (od == nullptr || od->n_elems == 0) return false;
  return b->particle_type == LS_HS_SPIN || (b->particle_type == LS_HS_SPINFUL_FERMION && od->fermionic);
}

static bool hamming_fixed(ls_hs_basis const* b) {
  if (b->particle_type == LS_HS_SPIN) return b->number_up >= 0;
  return b->number_particles >= 0;
}

static uint64_t low_ones(int k) { return k <= 0 ? 0 : (k >= 64 ? ~0ull : ((1ull << k) - 1)); }

// Basis.hs:734-774 for a spin / spinless-like description.
static void estimate_fixed(int n, int h, bool inversion, uint64_t* lo, uint64_t* hi) {
  if (h < 0) {
    *lo = 0;
    *hi = low_ones(n);
    return;
  }
  *lo = low_ones(h);
  const int sh = inversion ? n - h - 1 : n - h;
  *hi = (sh >= 64 || sh < 0) ? 0 : (low_ones(h) << sh);
}

static void state_estimates(ls_hs_basis const* b, uint64_t* lo, uint64_t* hi) {
  const int n = b->number_sites;
  if (b->particle_type == LS_HS_SPIN) {
    estimate_fixed(n, b->number_up, b->spin_inversion != 0, lo, hi);
  } else if (b->particle_type == LS_HS_SPINLESS_FERMION) {
    estimate_fixed(n, b->number_particles, false, lo, hi);
  } else {
    if (b->number_up >= 0) {
      uint64_t l0, h0, l1, h1;
      estimate_fixed(n, b->number_up, false, &l0, &h0);
      estimate_fixed(n, b->number_particles - b->number_up, false, &l1, &h1);
      *lo = (l1 << n) | l0;
      *hi = (h1 << n) | h0;
    } else {
      estimate_fixed(2 * n, b->number_particles, false, lo, hi);
    }
  }
}

static DeviceConstraint basis_constraint(ls_hs_basis const* b) {
  DeviceConstraint c;
  if (b->particle_type == LS_HS_SPIN) {
    if (b->number_up >= 0) {
      c.kind = 1;
      c.w0 = b->number_up;
    }
  } else if (b->particle_type == LS_HS_SPINLESS_FERMION) {
    if (b->number_particles >= 0) {
      c.kind = 1;
      c.w0 = b->number_particles;
    }
  } else {
    if (b->number_up >= 0) {
      c.kind = 2;
      c.half_bits = b->number_sites;
      c.w0 = b->number_up;
      c.w1 = b->number_particles - b->number_up;
    } else if (b->number_particles >= 0) {
      c.kind = 1;
      c.w0 = b->number_particles;
    }
  }
  return c;
}

// =================================================================================================
// Enumeration driver (StatesEnumeration.chpl:674-709)
// =================================================================================================
// Membership rule of projected enumeration: 0 keeps a state iff the reference's floating
// stabiliser sum is positive (StatesEnumeration.chpl:242-268 via is_representative), 1 iff its
// exact stabiliser has only trivial characters.  The two differ only in complex sectors, where the
// floating rule can keep rounding residue (norms ~1e-9 that are exactly zero).
static int g_enum_exact = 0;

extern "C" int ls_gpu_set_enumeration_rule(int exact) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const int previous = g_enum_exact;
  g_enum_exact = exact ? 1 : 0;
  return previous;
}

static int enumerate_into(ls_hs_basis const* b, uint64_t** d_out, int64_t* count) {
  EnumerateRequest req{};
  uint64_t lo, hi;
  state_estimates(b, &lo, &hi);
  req.lower = lo;
  req.upper = hi;
  req.number_sites = b->number_sites;
  req.spin_inversion = b->spin_inversion;
  req.hamming_fixed = hamming_fixed(b);
  req.reference_norm_rule = g_enum_exact ? 0 : 1;
  const OrbitData* od = basis_orbit(b);
  const DeviceGroup* g = nullptr;
  if (b->particle_type == LS_HS_SPIN) {
    if (has_permutations(b)) {
      req.mode = 0;
      g = orbit_device(od);
      if (g == nullptr) return LS_GPU_ERR_CUDA;
    } else {
      req.mode = 1;
    }
  } else if (b->particle_type == LS_HS_SPINFUL_FERMION && has_permutations(b)) {
    if (b->number_up < 0) return fail(LS_GPU_ERR_INVALID, "fermionic bases with lattice symmetries need fixed (N_up, N_down)");
    req.mode = 3;
    req.spin_inversion = 0;
    g = orbit_device(od);
    if (g == nullptr) return LS_GPU_ERR_CUDA;
  } else if (b->particle_type == LS_HS_SPINFUL_FERMION) {
    req.mode = b->number_up >= 0 ? 2 : 1;
    req.spin_inversion = 0;
  } else {
    req.mode = 1;
    req.spin_inversion = 0;
  }
  if (req.mode == 1 && b->particle_type == LS_HS_SPINFUL_FERMION) req.number_sites = 2 * b->number_sites;
  return enumerate_states(g, req, d_out, count, default_stream());
}

// Allocation-free enumeration for callers that cannot allocate device memory; see
// include/ls_gb300.h and the scratch description in basis.cu.  It builds the same request as
// enumerate_into but never uploads the group through cudaMalloc: the group tables are copied into
// the static scratch on every call.
extern "C" int ls_gpu_enumerate_noalloc(ls_hs_basis const* b, uint64_t* d_out, int64_t capacity,
                                        int64_t* count, void* stream) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (b == nullptr || count == nullptr) return fail(LS_GPU_ERR_INVALID, "basis and count must not be NULL");
  if (basis_number_bits(b) > 64) return fail(LS_GPU_ERR_INVALID, "bases with more than 64 bits are not supported");
  EnumerateRequest req{};
  uint64_t lo, hi;
  state_estimates(b, &lo, &hi);
  req.lower = lo;
  req.upper = hi;
  req.number_sites = b->number_sites;
  req.spin_inversion = b->spin_inversion;
  req.hamming_fixed = hamming_fixed(b);
  req.reference_norm_rule = g_enum_exact ? 0 : 1;
  const OrbitData* od = nullptr;
  if (b->particle_type == LS_HS_SPIN) {
    if (has_permutations(b)) {
      req.mode = 0;
      od = basis_orbit(b);
    } else {
      req.mode = 1;
    }
  } else if (b->particle_type == LS_HS_SPINFUL_FERMION && has_permutations(b)) {
    if (b->number_up < 0) return fail(LS_GPU_ERR_INVALID, "fermionic bases with lattice symmetries need fixed (N_up, N_down)");
    req.mode = 3;
    req.spin_inversion = 0;
    od = basis_orbit(b);
  } else if (b->particle_type == LS_HS_SPINFUL_FERMION) {
    req.mode = b->number_up >= 0 ? 2 : 1;
    req.spin_inversion = 0;
  } else {
    req.mode = 1;
    req.spin_inversion = 0;
  }
  if (req.mode == 1 && b->particle_type == LS_HS_SPINFUL_FERMION) req.number_sites = 2 * b->number_sites;
  return enumerate_states_noalloc(od, req, d_out, capacity, count, (cudaStream_t)stream);
}

extern "C" void ls_chpl_enumerate_representatives(ls_hs_basis* p, uint64_t lower, uint64_t upper,
                                                  chpl_external_array* dest) {
  (void)lower;  // the reference derives the range from the basis (StatesEnumeration.chpl:683-689)
  (void)upper;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (basis_number_bits(p) > 64) {
    set_error("bases with more than 64 bits are not yet implemented");
    report("ls_chpl_enumerate_representatives");
    return;
  }
  uint64_t* d = nullptr;
  int64_t n = 0;
  cudaStream_t s = default_stream();
  if (enumerate_into(p, &d, &n) != 0) {
    report("ls_chpl_enumerate_representatives");
    return;
  }
  uint64_t* h = nullptr;
  if (!cuda_ok(cudaMallocHost((void**)&h, std::max<int64_t>(n, 1) * 8), "cudaMallocHost(reps)") ||
      (n > 0 && !cuda_ok(cudaMemcpyAsync(h, d, (size_t)n * 8, cudaMemcpyDeviceToHost, s), "D2H reps")) ||
      !cuda_ok(cudaStreamSynchronize(s), "enumerate")) {
    cudaFree(d);
    report("ls_chpl_enumerate_representatives");
    return;
  }
  g_pending_device_reps[h] = d;
  dest->elts = h;
  dest->num_elts = (uint64_t)n;
  dest->freer = (void*)&free_pinned;
}

// reference.c:173-194
extern "C" void ls_hs_build_representatives(ls_hs_basis* basis, uint64_t lower, uint64_t upper) {
  ls_chpl_kernels const* kernels = ls_hs_internal_get_chpl_kernels();
  if (kernels->enumerate_states == nullptr)
    ls_hs_fatal_error(__func__, __LINE__, "enumerate_states kernel is NULL");
  if (basis->representatives.num_elts > 0) return;
  chpl_external_array arr{nullptr, 0, nullptr};
  kernels->enumerate_states(basis, lower, upper, &arr);
  if (arr.elts == nullptr && arr.num_elts == 0 && !g_last_error.empty()) {
    // error already reported through ls_hs_error
  }
  basis->representatives = arr;
  const int number_bits = basis_number_bits(basis);
  basis->kernels->state_index_data =
      ls_hs_create_state_index_binary_search_kernel_data(&basis->representatives, number_bits, 22);
  basis->kernels->state_index_kernel = &ls_hs_state_index_binary_search_kernel;
}

// reference.c:196-211
extern "C" void ls_hs_unchecked_set_representatives(ls_hs_basis* basis, chpl_external_array const* states,
                                                    int cache_bits) {
  if (basis->representatives.num_elts != 0)
    ls_hs_fatal_error(__func__, __LINE__, "representatives have already been set");
  if (basis->kernels == nullptr) ls_hs_fatal_error(__func__, __LINE__, "basis->kernels not set");
  if (basis->kernels->state_index_kernel != nullptr)
    ls_hs_fatal_error(__func__, __LINE__, "state_index_kernel has already been set");
  basis->representatives = *states;
  basis->kernels->state_index_data = ls_hs_create_state_index_binary_search_kernel_data(
      &basis->representatives, basis_number_bits(basis), cache_bits);
  basis->kernels->state_index_kernel = &ls_hs_state_index_binary_search_kernel;
}

extern "C" ptrdiff_t ls_hs_fixed_hamming_state_to_index(uint64_t basis_state) {
  return (ptrdiff_t)fixed_hamming_state_to_index(basis_state);
}
extern "C" uint64_t ls_hs_fixed_hamming_index_to_state(ptrdiff_t state_index, int hamming_weight) {
  return fixed_hamming_index_to_state((int64_t)state_index, hamming_weight);
}

// =================================================================================================
// Host term generation (reference.c:67-134 semantics)
// =================================================================================================
static inline double creal_of(ls_hs_scalar const& v) { return reinterpret_cast<const double*>(&v)[0]; }
static inline double cimag_of(ls_hs_scalar const& v) { return reinterpret_cast<const double*>(&v)[1]; }

extern "C" void ls_internal_operator_apply_diag_x1(ls_hs_operator const* op, ptrdiff_t batch_size,
                                                   uint64_t const* alphas, double* ys, double const* xs) {
  if (op->diag_terms == nullptr || op->diag_terms->number_terms == 0) {
    memset(ys, 0, (size_t)batch_size * sizeof(double));
    return;
  }
  ls_hs_nonbranching_terms const* t = op->diag_terms;
  for (ptrdiff_t i = 0; i < batch_size; ++i) {
    double acc = 0;
    const uint64_t a = alphas[i];
    for (int k = 0; k < t->number_terms; ++k) {
      if ((a & t->m[k]) == t->r[k]) {
        const int sign = 1 - 2 * (__builtin_popcountll(a & t->s[k]) % 2);
        const double factor = xs != nullptr ? sign * xs[i] : (double)sign;
        acc += creal_of(t->v[k]) * factor;
      }
    }
    ys[i] = acc;
  }
}

extern "C" void ls_internal_operator_apply_off_diag_x1(ls_hs_operator const* op, ptrdiff_t batch_size,
                                                       uint64_t const* alphas, uint64_t* betas,
                                                       ls_hs_scalar* coeffs, ptrdiff_t* offsets,
                                                       double const* xs) {
  if (op->off_diag_terms == nullptr || op->off_diag_terms->number_terms == 0) {
    memset(offsets, 0, (size_t)(batch_size + 1) * sizeof(ptrdiff_t));
    return;
  }
  ls_hs_nonbranching_terms const* t = op->off_diag_terms;
  double* c = reinterpret_cast<double*>(coeffs);
  offsets[0] = 0;
  ptrdiff_t off = 0;
  for (ptrdiff_t i = 0; i < batch_size; ++i) {
    const uint64_t a = alphas[i];
    for (int k = 0; k < t->number_terms; ++k) {
      if ((a & t->m[k]) == t->r[k]) {
        const int sign = 1 - 2 * (__builtin_popcountll(a & t->s[k]) % 2);
        const double factor = xs != nullptr ? sign * xs[i] : (double)sign;
        c[2 * off] = creal_of(t->v[k]) * factor;
        c[2 * off + 1] = cimag_of(t->v[k]) * factor;
        betas[off] = a ^ t->x[k];
        ++off;
      }
    }
    offsets[i + 1] = off;
  }
}

// BatchedOperator.chpl:298-316
extern "C" void ls_chpl_operator_apply_diag(ls_hs_operator* matrix, int64_t count, uint64_t* alphas,
                                            chpl_external_array* coeffs, int64_t num_tasks) {
  (void)num_tasks;
  if (basis_number_bits(matrix->basis) > 64) {
    ls_hs_error("bases with more than 64 bits are not yet implemented");
    return;
  }
  if (matrix->basis->requires_projection) {
    ls_hs_error("bases that require projection are not yet supported");
    return;
  }
  double* cs = (double*)malloc(std::max<int64_t>(count, 1) * sizeof(double));
  ls_internal_operator_apply_diag_x1(matrix, count, alphas, cs, nullptr);
  coeffs->elts = cs;
  coeffs->num_elts = (uint64_t)count;
  coeffs->freer = (void*)&free_malloced;
}

// BatchedOperator.chpl:318-357
extern "C" void ls_chpl_operator_apply_off_diag(ls_hs_operator* matrix, int64_t count, uint64_t* alphas,
                                                chpl_external_array* betas, chpl_external_array* coeffs,
                                                chpl_external_array* offsets, int64_t num_tasks) {
  (void)num_tasks;
  if (basis_number_bits(matrix->basis) > 64) {
    ls_hs_error("bases with more than 64 bits are not yet implemented");
    return;
  }
  const int nt = matrix->off_diag_terms ? matrix->off_diag_terms->number_terms : 0;
  ptrdiff_t* offs = (ptrdiff_t*)calloc((size_t)count + 1, sizeof(ptrdiff_t));
  if (nt != 0) {
    uint64_t* bs = (uint64_t*)malloc(std::max<int64_t>(count * nt, 1) * 8);
    ls_hs_scalar* cs = (ls_hs_scalar*)malloc(std::max<int64_t>(count * nt, 1) * 16);
    ls_internal_operator_apply_off_diag_x1(matrix, count, alphas, bs, cs, offs, nullptr);
    *betas = chpl_external_array{bs, (uint64_t)(count * nt), (void*)&free_malloced};
    *coeffs = chpl_external_array{cs, (uint64_t)(count * nt), (void*)&free_malloced};
  } else {
    *betas = chpl_external_array{nullptr, 0, nullptr};
    *coeffs = chpl_external_array{nullptr, 0, nullptr};
  }
  *offsets = chpl_external_array{offs, (uint64_t)count + 1, (void*)&free_malloced};
}

// =================================================================================================
// Operators on the device
// =================================================================================================
namespace {

struct TermTable {
  int n = 0;
  std::vector<uint64_t> m, l, r, x, s;
  std::vector<double> v;  // interleaved
};

struct DeviceTermSet {
  void* block = nullptr;
  DeviceTerms terms;
};

struct OperatorCache {
  TermTable off, diag;             // host copies (validated on every use)
  DeviceTermSet fwd_off, adj_off, fwd_diag, adj_diag;
  std::vector<int32_t> coupling;   // optional, per term (off then diag)
  int32_t* d_coupling = nullptr;
};

std::unordered_map<const ls_hs_operator*, OperatorCache*> g_ops;

TermTable read_terms(ls_hs_nonbranching_terms const* t) {
  TermTable tt;
  if (t == nullptr) return tt;
  tt.n = t->number_terms;
  tt.m.assign(t->m, t->m + tt.n);
  tt.l.assign(t->l, t->l + tt.n);
  tt.r.assign(t->r, t->r + tt.n);
  tt.x.assign(t->x, t->x + tt.n);
  tt.s.assign(t->s, t->s + tt.n);
  const double* v = reinterpret_cast<const double*>(t->v);
  tt.v.assign(v, v + 2 * (size_t)tt.n);
  return tt;
}

bool same_terms(const TermTable& a, ls_hs_nonbranching_terms const* t) {
  const int n = t ? t->number_terms : 0;
  if (a.n != n) return false;
  if (n == 0) return true;
  return memcmp(a.m.data(), t->m, n * 8) == 0 && memcmp(a.l.data(), t->l, n * 8) == 0 &&
         memcmp(a.r.data(), t->r, n * 8) == 0 && memcmp(a.x.data(), t->x, n * 8) == 0 &&
         memcmp(a.s.data(), t->s, n * 8) == 0 &&
         memcmp(a.v.data(), reinterpret_cast<const double*>(t->v), (size_t)n * 16) == 0;
}

// T^dagger: conj(v) (-1)^popcount(x & s), l and r exchanged.
TermTable adjoint_terms(const TermTable& t) {
  TermTable a = t;
  for (int k = 0; k < t.n; ++k) {
    std::swap(a.l[k], a.r[k]);
    double sign = (__builtin_popcountll(t.x[k] & t.s[k]) & 1) ? -1.0 : 1.0;
    a.v[2 * k] = sign * t.v[2 * k];
    a.v[2 * k + 1] = -sign * t.v[2 * k + 1];
  }
  return a;
}

// Whether applying a term can change a particle number that the basis conserves.
bool term_breaks_constraint(const DeviceConstraint& c, uint64_t l, uint64_t r) {
  if (c.kind == 0) return false;
  if (c.kind == 1) return __builtin_popcountll(l) != __builtin_popcountll(r);
  const uint64_t lo = c.half_bits >= 64 ? ~0ull : ((1ull << c.half_bits) - 1);
  return __builtin_popcountll(l & lo) != __builtin_popcountll(r & lo) ||
         __builtin_popcountll(l & ~lo) != __builtin_popcountll(r & ~lo);
}

// Device layout: v (double2, 16-byte aligned) first, then m, l, r, x, s (uint64), xinfo (uint32).
int upload_terms(const TermTable& t, const DeviceConstraint& cons, DeviceTermSet* out) {
  const size_t n = (size_t)std::max(t.n, 1);
  const size_t bytes = n * (16 + 5 * 8 + 4);
  std::vector<uint8_t> host(bytes, 0);
  uint8_t* p = host.data();
  auto put = [&](const void* src, size_t sz, size_t off) {
    if (t.n > 0) memcpy(p + off, src, sz);
  };
  const size_t ov = 0, om = n * 16, ol = om + n * 8, orr = ol + n * 8, ox = orr + n * 8, os = ox + n * 8;
  const size_t oi = os + n * 8;
  put(t.v.data(), t.n * 16, ov);
  put(t.m.data(), t.n * 8, om);
  put(t.l.data(), t.n * 8, ol);
  put(t.r.data(), t.n * 8, orr);
  put(t.x.data(), t.n * 8, ox);
  put(t.s.data(), t.n * 8, os);
  std::vector<uint32_t> xinfo(n, 0);
  int all_two = t.n > 0 ? 1 : 0;
  for (int k = 0; k < t.n; ++k) {
    const uint64_t x = t.x[k];
    const int cnt = __builtin_popcountll(x);
    const int lo = x ? __builtin_ctzll(x) : 0;
    const int hi = x ? 63 - __builtin_clzll(x) : 0;
    uint32_t info = (uint32_t)lo | ((uint32_t)hi << 8) | ((uint32_t)cnt << 16);
    if (term_breaks_constraint(cons, t.l[k], t.r[k])) info |= kTermNeedsCheck;
    xinfo[k] = info;
    if (cnt != 2 || (info & kTermNeedsCheck)) all_two = 0;
  }
  put(xinfo.data(), t.n * 4, oi);
  out->terms.all_two_site = all_two;
  if (!cuda_ok(cudaMalloc(&out->block, bytes), "cudaMalloc(terms)")) return LS_GPU_ERR_CUDA;
  if (!cuda_ok(cudaMemcpy(out->block, host.data(), bytes, cudaMemcpyHostToDevice), "upload terms"))
    return LS_GPU_ERR_CUDA;
  uint8_t* d = (uint8_t*)out->block;
  out->terms.n = t.n;
  out->terms.v = (const double2*)(d + ov);
  out->terms.m = (const uint64_t*)(d + om);
  out->terms.l = (const uint64_t*)(d + ol);
  out->terms.r = (const uint64_t*)(d + orr);
  out->terms.x = (const uint64_t*)(d + ox);
  out->terms.s = (const uint64_t*)(d + os);
  out->terms.xinfo = (const uint32_t*)(d + oi);
  return 0;
}

void free_cache(OperatorCache* c) {
  for (DeviceTermSet* s : {&c->fwd_off, &c->adj_off, &c->fwd_diag, &c->adj_diag})
    if (s->block) cudaFree(s->block);
  if (c->d_coupling) cudaFree(c->d_coupling);
  delete c;
}

OperatorCache* operator_cache(const ls_hs_operator* op) {
  auto it = g_ops.find(op);
  if (it != g_ops.end()) {
    OperatorCache* c = it->second;
    if (same_terms(c->off, op->off_diag_terms) && same_terms(c->diag, op->diag_terms)) return c;
    free_cache(c);
    g_ops.erase(it);
  }
  OperatorCache* c = new OperatorCache();
  c->off = read_terms(op->off_diag_terms);
  c->diag = read_terms(op->diag_terms);
  const DeviceConstraint cons = op->basis ? basis_constraint(op->basis) : DeviceConstraint{};
  if (upload_terms(c->off, cons, &c->fwd_off) || upload_terms(adjoint_terms(c->off), cons, &c->adj_off) ||
      upload_terms(c->diag, cons, &c->fwd_diag) || upload_terms(adjoint_terms(c->diag), cons, &c->adj_diag)) {
    free_cache(c);
    return nullptr;
  }
  g_ops[op] = c;
  return c;
}

int ensure_norms(IndexData* ix, const OrbitData* od) {
  if (ix->d_norms != nullptr && ix->norms_for == od) return 0;
  cudaStream_t s = default_stream();
  // one allocation: norms [n] | inverse norms [n]
  const int64_t n = std::max<int64_t>(ix->n_states, 1);
  if (ix->d_norms == nullptr &&
      !cuda_ok(cudaMalloc((void**)&ix->d_norms, (size_t)n * 2 * 8), "cudaMalloc(norms)"))
    return LS_GPU_ERR_CUDA;
  int rc;
  if (od != nullptr && od->n_elems > 0) {
    const DeviceGroup* dg = orbit_device(od);
    rc = dg ? launch_orbit_norms(*dg, ix->n_states, ix->d_reps, ix->d_norms, s) : LS_GPU_ERR_CUDA;
  } else {
    std::vector<double> ones((size_t)n, 1.0);
    rc = cuda_ok(cudaMemcpyAsync(ix->d_norms, ones.data(), ones.size() * 8, cudaMemcpyHostToDevice, s),
                 "norms") ? 0 : LS_GPU_ERR_CUDA;
  }
  if (rc == 0) rc = launch_inverse_norms(ix->d_norms, ix->n_states, ix->d_norms + n, s);
  // The norms are computed on the library's stream but read by kernels on the caller's stream:
  // finish them before any caller can launch.
  if (rc == 0) rc = cuda_ok(cudaStreamSynchronize(s), "orbit norms") ? 0 : LS_GPU_ERR_CUDA;
  if (rc == 0) {
    ix->norms_for = od;
    ix->dev.norms = ix->d_norms;
    ix->dev.inv_norms = ix->d_norms + n;
  }
  return rc;
}

// Builds the kernel-side description of y = op x (adjoint: y = op^dagger x).
int make_problem(ls_hs_operator const* op, bool adjoint, MatvecProblem* p) {
  ls_hs_basis const* b = op->basis;
  if (b == nullptr) return fail(LS_GPU_ERR_INVALID, "operator has no basis");
  if (basis_number_bits(b) > 64) return fail(LS_GPU_ERR_INVALID, "bases with more than 64 bits are not yet implemented");
  IndexData* ix = basis_index(b);
  if (ix == nullptr) return fail(LS_GPU_ERR_NOT_BUILT, "basis is not built on the GPU");
  const OrbitData* od = basis_orbit(b);
  OperatorCache* c = operator_cache(op);
  if (c == nullptr) return LS_GPU_ERR_CUDA;
  p->projection = !b->requires_projection ? 0 : (has_permutations(b) ? 2 : 1);
  if (p->projection == 1 && b->spin_inversion == 0) return fail(LS_GPU_ERR_INVALID, "projection without symmetries");
  if (ensure_norms(ix, p->projection == 2 ? od : nullptr) != 0) return LS_GPU_ERR_CUDA;
  p->group = DeviceGroup{};
  if (p->projection == 2) {
    const DeviceGroup* dg = orbit_device(od);
    if (dg == nullptr) return LS_GPU_ERR_CUDA;
    p->group = *dg;
  }
  p->group.spin_inversion = b->spin_inversion;
  p->group.n_bits = basis_number_bits(b);
  p->group.flip = low_ones(b->number_sites);
  p->index = ix->dev;
  // DistributedMatrixVector.chpl:105-113: identity index on one locale.
  p->index.identity = b->state_index_is_identity ? 1 : 0;
  // Without permutations a fixed-weight spin basis is a contiguous combinadic range starting at
  // rank 0 (all states, or all states below the flipped maximum under spin inversion).
  if (p->projection != 2 && !p->index.identity && b->particle_type == LS_HS_SPIN && b->number_up >= 0) {
    p->index.combinadic = 1;
    p->index.rank_base = 0;
  }
  p->constraint = basis_constraint(b);
  p->off = adjoint ? c->adj_off.terms : c->fwd_off.terms;
  p->diag = adjoint ? c->adj_diag.terms : c->fwd_diag.terms;
  p->off.coupling = p->diag.coupling = c->d_coupling;
  p->n_rows = ix->n_states;
  // Real matrix elements: real term coefficients and real characters.  Characters are
  // cos/sin(-2 pi phi) in floating point (Group.hs:115-116), so sectors such as (pi, pi) carry
  // imaginary parts of order 1e-16; below 1e-14 they are treated as zero here (the dropped terms
  // are below 1e-15 of the result).
  bool real = true;
  for (int t = 0; t < c->off.n && real; ++t) real = c->off.v[2 * t + 1] == 0.0;
  if (p->projection == 2 && od != nullptr)
    for (int e = 0; e < od->n_elems && real; ++e) real = std::fabs(od->chars_im[e]) <= 1e-14;
  p->real_elements = real ? 1 : 0;
  return 0;
}

int read_and_clear_error(cudaStream_t s) {
  int h[4] = {0, 0, 0, 0};
  int* d = device_error_word();
  if (!cuda_ok(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s), "read error word") ||
      !cuda_ok(cudaMemsetAsync(d, 0, sizeof(h), s), "clear error word") ||
      !cuda_ok(cudaStreamSynchronize(s), "matvec"))
    return LS_GPU_ERR_CUDA;
  if (h[0] != 0)
    return fail(LS_GPU_ERR_BASIS,
                "a generated basis state does not belong to the basis (the operator does not conserve "
                "the basis' particle numbers)");
  if (h[1] != 0)
    return fail(LS_GPU_ERR_CUDA, "a tensor-core block product gave up waiting for its MMAs (results invalid)");
  return 0;
}

}  // namespace

// Writes one word in every page of [p, p + bytes) from several host threads, so that the pages
// of a freshly allocated output are mapped (faulted in and zeroed by the OS) while the GPU
// computes, instead of during the device-to-host copy.  The range is an output: its contents are
// overwritten afterwards.
static void prefault_output(void* p, size_t bytes) {
  const long page = sysconf(_SC_PAGESIZE);
  const size_t step = page > 0 ? (size_t)page : 4096;
  const size_t pages = (bytes + step - 1) / step;
  if (pages < 256) return;  // small outputs: not worth the threads
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(std::min<size_t>(hw, 16), pages / 64);
  auto work = [=](size_t t) {
    volatile unsigned char* base = (volatile unsigned char*)p;
    for (size_t q = t; q < pages; q += nt) base[q * step] = 0;
  };
  std::vector<std::thread> threads;
  for (size_t t = 1; t < nt; ++t) threads.emplace_back(work, t);
  work(0);
  for (auto& th : threads) th.join();
}

// DistributedMatrixVector.chpl:1090-1105: y = H x on host arrays.  The reference accepts one real
// vector; here num_vectors >= 1 vectors stored one after the other (x[v * D + i]) go through one
// orbit scan (they are transposed on the device to the kernels' [D][k] layout).
extern "C" void ls_chpl_matrix_vector_product(ls_hs_operator* matrix, int num_vectors, double const* x,
                                              double* y) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (basis_number_bits(matrix->basis) > 64) {
    ls_hs_error("bases with more than 64 bits are not yet implemented");
    return;
  }
  if (num_vectors < 1) {
    ls_hs_error("the number of vectors must be positive");
    return;
  }
  cudaStream_t s = default_stream();
  StageScope call_stage("io.call", s);
  MatvecProblem p;
  int rc = make_problem(matrix, false, &p);
  if (rc != 0) {
    report("ls_chpl_matrix_vector_product");
    return;
  }
  const int64_t n = p.n_rows;
  const int k = num_vectors;
  const size_t bytes = (size_t)std::max<int64_t>(n, 1) * k * 8;
  double* d_x = (double*)scratch(bytes, 4);
  double* d_y = (double*)scratch(bytes, 5);
  double* d_xt = k > 1 ? (double*)scratch(bytes, 8) : d_x;
  double* d_yt = k > 1 ? (double*)scratch(bytes, 9) : d_y;
  if (!d_x || !d_y || !d_xt || !d_yt) {
    report("ls_chpl_matrix_vector_product");
    return;
  }
  if (n > 0) {
    const size_t vbytes = (size_t)n * k * 8;
    // x is pinned for the copy when the system allows it (a DMA at full speed; a pageable copy of
    // a large host array can be staged far slower) and unpinned before returning
    bool pinned_x = false;
    if (vbytes >= (1u << 20)) {
      // the default flags need writable pages; read-only registration where those fail
      pinned_x = cudaHostRegister((void*)x, vbytes, cudaHostRegisterDefault) == cudaSuccess;
      if (!pinned_x) {
        cudaGetLastError();
        pinned_x = cudaHostRegister((void*)x, vbytes, cudaHostRegisterReadOnly) == cudaSuccess;
      }
      if (!pinned_x) cudaGetLastError();  // not registered (already pinned, or unsupported): plain copy
    }
    const bool overlap = (const char*)y < (const char*)x + vbytes && (const char*)x < (const char*)y + vbytes;
    {
      StageScope stage("io.h2d", s);
      if (!cuda_ok(cudaMemcpyAsync(d_x, x, vbytes, cudaMemcpyHostToDevice, s), "H2D x")) rc = LS_GPU_ERR_CUDA;
    }
    if (rc == 0 && k > 1) {
      StageScope stage("io.transpose", s);
      rc = launch_transpose(d_x, d_xt, k, n, s);
    }
    if (rc == 0) rc = launch_matvec(p, Scalar::Real, k, d_xt, k, d_yt, k, device_error_word(), s);
    if (rc == 0 && k > 1) {
      StageScope stage("io.transpose", s);
      rc = launch_transpose(d_yt, d_y, n, k, s);
    }
    // the host maps y's pages while the GPU computes (the copy below waits for the kernels); not
    // when y overlaps x, whose copy may still be in flight
    if (rc == 0 && !overlap) {
      StageScope stage("io.prefault", s);
      prefault_output(y, vbytes);
    }
    if (rc == 0) {
      StageScope stage("io.d2h", s);
      if (!cuda_ok(cudaMemcpyAsync(y, d_y, vbytes, cudaMemcpyDeviceToHost, s), "D2H y")) rc = LS_GPU_ERR_CUDA;
    }
    if (rc == 0) rc = read_and_clear_error(s);
    if (pinned_x) {
      if (rc != 0) cudaStreamSynchronize(s);  // the copy of x has finished before x is unpinned
      cudaHostUnregister((void*)x);
    }
  }
  if (rc != 0) report("ls_chpl_matrix_vector_product");
}

// =================================================================================================
// Additive API
// =================================================================================================
extern "C" int ls_gpu_basis_info(ls_hs_basis const* basis, int64_t* number_states,
                                 uint64_t const** d_representatives, double const** d_norms) {
  std::lock_guard<std::mutex> lock(g_mutex);
  IndexData* ix = basis_index(basis);
  if (ix == nullptr) return fail(LS_GPU_ERR_NOT_BUILT, "basis is not built on the GPU");
  const OrbitData* od = has_permutations(basis) ? basis_orbit(basis) : nullptr;
  if (ensure_norms(ix, od) != 0) return LS_GPU_ERR_CUDA;
  if (number_states) *number_states = ix->n_states;
  if (d_representatives) *d_representatives = ix->d_reps;
  if (d_norms) *d_norms = ix->d_norms;
  return 0;
}

// Stream-ordered: enqueues the kernels and returns; a generated state outside the basis is
// recorded in the device error word and reported by ls_gpu_check_errors.
static int gpu_matvec(ls_hs_operator const* op, Scalar sc, int k, double const* d_x, int64_t ldx,
                      double* d_y, int64_t ldy, int adjoint, void* stream,
                      unsigned long long* nnz_counter = nullptr) {
  if (k < 0 || ldx < k || ldy < k) return fail(LS_GPU_ERR_INVALID, "invalid k / leading dimension");
  std::lock_guard<std::mutex> lock(g_mutex);
  MatvecProblem p;
  int rc = make_problem(op, adjoint != 0, &p);
  if (rc != 0) return rc;
  p.nnz_counter = nnz_counter;
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream (CUDA convention)
  return launch_matvec(p, sc, k, d_x, ldx, d_y, ldy, device_error_word(), s);
}

extern "C" int ls_gpu_check_errors(void* stream);

// Times the matvec of `op` on k complex right-hand sides for every (threads per block, grid
// waves) pair of a small table and installs the fastest with ls_gpu_set_matvec_config.
extern "C" int ls_gpu_autotune_matvec(ls_hs_operator const* op, int k, int* best_threads, int* best_waves,
                                      double* best_ms) {
  if (k < 1) return fail(LS_GPU_ERR_INVALID, "k must be positive");
  int64_t n = 0;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    IndexData* ix = op && op->basis ? basis_index(op->basis) : nullptr;
    if (ix == nullptr) return fail(LS_GPU_ERR_NOT_BUILT, "basis is not built on the GPU");
    n = ix->n_states;
  }
  cudaStream_t s = default_stream();
  double* d_x = nullptr;
  double* d_y = nullptr;
  const size_t bytes = (size_t)std::max<int64_t>(n, 1) * k * 16;
  if (!cuda_ok(cudaMalloc((void**)&d_x, bytes), "alloc") || !cuda_ok(cudaMalloc((void**)&d_y, bytes), "alloc")) {
    cudaFree(d_x);
    return LS_GPU_ERR_CUDA;
  }
  cudaMemsetAsync(d_x, 0, bytes, s);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // threads per CTA (each kernel clamps to its own maximum; 0 = that maximum) x grid waves
  const int threads_choices[] = {0, 768, 512};
  const int wave_choices[] = {1, 2, 4, 8};
  double best = 1e300;
  int bt = 0, bw = 4, rc = 0;
  for (int th : threads_choices) {
    for (int wv : wave_choices) {
      set_matvec_config(th, wv);
      rc = gpu_matvec(op, Scalar::Complex, k, d_x, k, d_y, k, 0, s);  // warm-up / validation
      if (rc != 0) break;
      cudaEventRecord(e0, s);
      rc = gpu_matvec(op, Scalar::Complex, k, d_x, k, d_y, k, 0, s);
      cudaEventRecord(e1, s);
      if (rc != 0 || !cuda_ok(cudaEventSynchronize(e1), "autotune")) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        bt = th;
        bw = wv;
      }
    }
    if (rc != 0) break;
  }
  set_matvec_config(bt, bw);
  // right-hand-side tile: for k >= 8, one launch of 16 columns against two of 8 (or four of 4)
  int btile = 16;
  if (rc == 0 && k >= 8) {
    double tbest = 1e300;
    for (int tile : {16, 8, 4}) {
      if (tile > k && tile != 4) continue;
      set_matvec_rhs_tile(tile);
      rc = gpu_matvec(op, Scalar::Complex, k, d_x, k, d_y, k, 0, s);
      if (rc != 0) break;
      cudaEventRecord(e0, s);
      rc = gpu_matvec(op, Scalar::Complex, k, d_x, k, d_y, k, 0, s);
      cudaEventRecord(e1, s);
      if (rc != 0 || !cuda_ok(cudaEventSynchronize(e1), "autotune")) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < tbest) {
        tbest = ms;
        btile = tile;
      }
    }
    if (tbest < best) best = tbest;
  }
  set_matvec_rhs_tile(btile);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d_x);
  cudaFree(d_y);
  if (rc == 0) rc = ls_gpu_check_errors(s);
  if (best_threads) *best_threads = bt;
  if (best_waves) *best_waves = bw;
  if (best_ms) *best_ms = best;
  return rc;
}

extern "C" int ls_gpu_check_errors(void* stream) {
  std::lock_guard<std::mutex> lock(g_mutex);
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream (CUDA convention)
  return read_and_clear_error(s);
}

extern "C" int ls_gpu_set_tracing(int on) {
  set_tracing(on != 0);
  return 0;
}

extern "C" int ls_gpu_trace_report(char* buffer, size_t size, int reset) {
  return trace_report(buffer, size, reset != 0);
}

extern "C" int ls_gpu_matvec_kernel_info(ls_hs_operator const* op, int* form, int* slots_per_lane) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (op == nullptr || form == nullptr || slots_per_lane == nullptr)
    return fail(LS_GPU_ERR_INVALID, "operator and outputs must not be NULL");
  MatvecProblem p;
  const int rc = make_problem(op, false, &p);
  if (rc != 0) return rc;
  *form = matvec_kernel_form(p, slots_per_lane);
  return 0;
}

extern "C" int ls_gpu_count_nonzeros(ls_hs_operator const* op, int64_t* nnz) {
  int64_t n = 0;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    IndexData* ix = op && op->basis ? basis_index(op->basis) : nullptr;
    if (ix == nullptr) return fail(LS_GPU_ERR_NOT_BUILT, "basis is not built on the GPU");
    n = ix->n_states;
  }
  cudaStream_t s = default_stream();
  double* d_x = nullptr;
  double* d_y = nullptr;
  unsigned long long* d_cnt = nullptr;
  int rc = 0;
  if (!cuda_ok(cudaMalloc((void**)&d_x, std::max<int64_t>(n, 1) * 8), "alloc") ||
      !cuda_ok(cudaMalloc((void**)&d_y, std::max<int64_t>(n, 1) * 8), "alloc") ||
      !cuda_ok(cudaMalloc((void**)&d_cnt, 8), "alloc")) {
    rc = LS_GPU_ERR_CUDA;
  }
  if (rc == 0) {
    cudaMemsetAsync(d_x, 0, std::max<int64_t>(n, 1) * 8, s);
    cudaMemsetAsync(d_cnt, 0, 8, s);
    rc = gpu_matvec(op, Scalar::Real, 1, d_x, 1, d_y, 1, 0, s, d_cnt);
  }
  unsigned long long h = 0;
  if (rc == 0 && (!cuda_ok(cudaMemcpyAsync(&h, d_cnt, 8, cudaMemcpyDeviceToHost, s), "read nnz") ||
                  !cuda_ok(cudaStreamSynchronize(s), "count")))
    rc = LS_GPU_ERR_CUDA;
  if (rc == 0) rc = ls_gpu_check_errors(s);
  cudaFree(d_x);
  cudaFree(d_y);
  cudaFree(d_cnt);
  if (rc == 0 && nnz) *nnz = (int64_t)h;
  return rc;
}

extern "C" int ls_gpu_matvec_c128(ls_hs_operator const* op, int k, double const* d_x, int64_t ldx,
                                  double* d_y, int64_t ldy, int adjoint, void* stream) {
  return gpu_matvec(op, Scalar::Complex, k, d_x, ldx, d_y, ldy, adjoint, stream);
}

extern "C" int ls_gpu_matvec_f64(ls_hs_operator const* op, int k, double const* d_x, int64_t ldx,
                                 double* d_y, int64_t ldy, int adjoint, void* stream) {
  return gpu_matvec(op, Scalar::Real, k, d_x, ldx, d_y, ldy, adjoint, stream);
}

extern "C" int ls_gpu_state_info(ls_hs_basis const* basis, int64_t batch, uint64_t const* d_alphas,
                                 uint64_t* d_betas, double* d_characters, double* d_norms, void* stream) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const OrbitData* od = basis_orbit(basis);
  if (od == nullptr || od->n_elems == 0) return fail(LS_GPU_ERR_INVALID, "basis has no symmetry group on the GPU");
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream (CUDA convention)
  const DeviceGroup* dg = orbit_device(od);
  if (dg == nullptr) return LS_GPU_ERR_CUDA;
  return launch_state_info(*dg, batch, d_alphas, d_betas, (double2*)d_characters, d_norms, 8, s);
}

extern "C" int ls_gpu_is_representative(ls_hs_basis const* basis, int64_t batch, uint64_t const* d_alphas,
                                        uint8_t* d_flags, double* d_norms, void* stream) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const OrbitData* od = basis_orbit(basis);
  if (od == nullptr || od->n_elems == 0) return fail(LS_GPU_ERR_INVALID, "basis has no symmetry group on the GPU");
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream (CUDA convention)
  const DeviceGroup* dg = orbit_device(od);
  if (dg == nullptr) return LS_GPU_ERR_CUDA;
  return launch_is_representative(*dg, batch, d_alphas, d_flags, d_norms, 4, s);
}

extern "C" int ls_gpu_state_index(ls_hs_basis const* basis, int64_t batch, uint64_t const* d_alphas,
                                  int64_t* d_indices, void* stream) {
  std::lock_guard<std::mutex> lock(g_mutex);
  IndexData* ix = basis_index(basis);
  if (ix == nullptr) return fail(LS_GPU_ERR_NOT_BUILT, "basis is not built on the GPU");
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream (CUDA convention)
  return launch_state_index(ix->dev, batch, d_alphas, d_indices, s);
}

// Frees the device copies of an operator's term tables (uploaded on first use, keyed by the
// ls_hs_operator address).  Call it before the operator's memory is released or reused; sector
// plans that use the operator fail to run afterwards instead of reading freed tables.
extern "C" void ls_gpu_release_operator(ls_hs_operator const* op) {
  std::lock_guard<std::mutex> lock(g_mutex);
  auto it = g_ops.find(op);
  if (it == g_ops.end()) return;
  free_cache(it->second);
  g_ops.erase(it);
}

// BatchedOperator.chpl:298-357 / reference.c:67-135 on device batches (see apply.cu).
extern "C" int ls_gpu_operator_apply_diag(ls_hs_operator const* op, int64_t count, uint64_t const* d_alphas,
                                          double* d_ys, void* stream) {
  if (op == nullptr || count < 0 || (count > 0 && (d_alphas == nullptr || d_ys == nullptr)))
    return fail(LS_GPU_ERR_INVALID, "invalid arguments");
  std::lock_guard<std::mutex> lock(g_mutex);
  OperatorCache* c = operator_cache(op);
  if (c == nullptr) return LS_GPU_ERR_CUDA;
  return launch_apply_diag(c->fwd_diag.terms, count, d_alphas, d_ys, (cudaStream_t)stream);
}

extern "C" int ls_gpu_operator_apply_off_diag(ls_hs_operator const* op, int64_t count, uint64_t const* d_alphas,
                                              uint64_t* d_betas, double* d_coeffs, int64_t* d_offsets,
                                              void* stream) {
  if (op == nullptr || count < 0 || d_offsets == nullptr || (count > 0 && d_alphas == nullptr))
    return fail(LS_GPU_ERR_INVALID, "invalid arguments");
  std::lock_guard<std::mutex> lock(g_mutex);
  OperatorCache* c = operator_cache(op);
  if (c == nullptr) return LS_GPU_ERR_CUDA;
  if (c->off.n > 0 && count > 0 && (d_betas == nullptr || d_coeffs == nullptr))
    return fail(LS_GPU_ERR_INVALID, "betas and coeffs need count * number_off_diag_terms entries");
  return launch_apply_off_diag(c->fwd_off.terms, count, d_alphas, d_betas, d_coeffs, d_offsets,
                               (cudaStream_t)stream);
}

extern "C" int ls_gpu_coupling_inner_products(ls_hs_operator const* op, int n_couplings,
                                              int32_t const* term_coupling, double const* d_g,
                                              double const* d_x, double* d_out, void* stream) {
  if (op == nullptr || term_coupling == nullptr || d_g == nullptr || d_x == nullptr || d_out == nullptr)
    return fail(LS_GPU_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lock(g_mutex);
  MatvecProblem p;
  int rc = make_problem(op, false, &p);
  if (rc != 0) return rc;
  OperatorCache* c = g_ops[op];
  const int n_terms = c->off.n + c->diag.n;
  for (int t = 0; t < n_terms; ++t)
    if (term_coupling[t] < 0 || term_coupling[t] >= n_couplings)
      return fail(LS_GPU_ERR_INVALID, "term coupling id out of range");
  if (c->d_coupling == nullptr || c->coupling.size() != (size_t)n_terms ||
      memcmp(c->coupling.data(), term_coupling, (size_t)n_terms * 4) != 0) {
    if (c->d_coupling) cudaFree(c->d_coupling);
    c->d_coupling = nullptr;
    c->coupling.assign(term_coupling, term_coupling + n_terms);
    if (!cuda_ok(cudaMalloc((void**)&c->d_coupling, (size_t)std::max(n_terms, 1) * 4), "cudaMalloc(couplings)") ||
        !cuda_ok(cudaMemcpy(c->d_coupling, c->coupling.data(), (size_t)n_terms * 4, cudaMemcpyHostToDevice),
                 "upload couplings")) {
      c->coupling.clear();
      return LS_GPU_ERR_CUDA;
    }
  }
  p.off.coupling = c->d_coupling;
  p.diag.coupling = c->d_coupling + c->off.n;
  return launch_coupling_products(p, n_couplings, d_g, d_x, d_out, device_error_word(), (cudaStream_t)stream);
}

namespace {
constexpr uint32_t kPlanMagic = 0x504c414eu;  // "PLAN"
struct SectorPlanHandle {
  uint32_t magic = kPlanMagic;
  int device = 0;
  std::vector<const ls_hs_operator*> ops;
  std::vector<OperatorCache*> caches;
  SectorPlan* plan = nullptr;
};

// Whether sector i can share sector 0's shared-memory tables in one batched launch.
bool sectors_share_tables(ls_hs_operator const* a, ls_hs_operator const* b, const MatvecProblem& pa,
                          const MatvecProblem& pb) {
  if (pa.projection != 2 || pb.projection != 2) return false;
  if (pa.group.n_bits != pb.group.n_bits || pa.group.gpl != pb.group.gpl || pa.group.n_elems != pb.group.n_elems)
    return false;
  if ((pa.group.spin_inversion != 0) != (pb.group.spin_inversion != 0)) return false;
  const DeviceConstraint &ca = pa.constraint, &cb = pb.constraint;
  if (ca.kind != cb.kind || ca.half_bits != cb.half_bits || ca.w0 != cb.w0 || ca.w1 != cb.w1) return false;
  const OrbitData* oa = basis_orbit(a->basis);
  const OrbitData* ob = basis_orbit(b->basis);
  if (oa == nullptr || ob == nullptr || oa->gpl != ob->gpl || oa->gpl == 0) return false;
  const size_t bytes = (size_t)oa->n_bits * 32 * oa->gpl * 8;
  if (oa->host_block.size() < oa->off_onehot_packed + bytes || ob->host_block.size() < ob->off_onehot_packed + bytes)
    return false;
  if (memcmp(oa->host_block.data() + oa->off_onehot_packed, ob->host_block.data() + ob->off_onehot_packed, bytes) != 0)
    return false;
  OperatorCache* c = g_ops[a];
  return c != nullptr && same_terms(c->off, b->off_diag_terms) && same_terms(c->diag, b->diag_terms);
}
}  // namespace

extern "C" int ls_gpu_sector_plan_create(int n_sectors, ls_hs_operator const* const* ops, int k,
                                         double const* const* d_x, int64_t ldx, double* const* d_y,
                                         int64_t ldy, int adjoint, void** plan) {
  if (plan == nullptr) return fail(LS_GPU_ERR_INVALID, "plan must not be NULL");
  *plan = nullptr;
  if (n_sectors < 1 || ops == nullptr || d_x == nullptr || d_y == nullptr)
    return fail(LS_GPU_ERR_INVALID, "need at least one sector with operators and vectors");
  if (k < 1 || ldx < k || ldy < k) return fail(LS_GPU_ERR_INVALID, "invalid k / leading dimension");
  std::lock_guard<std::mutex> lock(g_mutex);
  std::vector<MatvecProblem> problems(n_sectors);
  SectorPlanHandle* h = new SectorPlanHandle();
  cudaGetDevice(&h->device);
  for (int i = 0; i < n_sectors; ++i) {
    if (ops[i] == nullptr) {
      delete h;
      return fail(LS_GPU_ERR_INVALID, "NULL operator in the sector list");
    }
    const int rc = make_problem(ops[i], adjoint != 0, &problems[i]);
    if (rc != 0) {
      delete h;
      return rc;
    }
    h->ops.push_back(ops[i]);
    h->caches.push_back(g_ops[ops[i]]);
  }
  bool share = true;
  for (int i = 1; i < n_sectors && share; ++i)
    share = sectors_share_tables(ops[0], ops[i], problems[0], problems[i]);
  std::vector<const double*> xs(d_x, d_x + n_sectors);
  std::vector<double*> ys(d_y, d_y + n_sectors);
  const int rc = sector_plan_build(problems, share, k, xs, ldx, ys, ldy, &h->plan);
  if (rc != 0) {
    delete h;
    return rc;
  }
  *plan = h;
  return 0;
}

extern "C" int ls_gpu_sector_plan_is_batched(void const* plan) {
  const SectorPlanHandle* h = (const SectorPlanHandle*)plan;
  if (h == nullptr || h->magic != kPlanMagic) return fail(LS_GPU_ERR_INVALID, "not a sector plan");
  return sector_plan_batched(h->plan) ? 1 : 0;
}

extern "C" int ls_gpu_sector_plan_run(void const* plan, void* stream) {
  const SectorPlanHandle* h = (const SectorPlanHandle*)plan;
  if (h == nullptr || h->magic != kPlanMagic) return fail(LS_GPU_ERR_INVALID, "not a sector plan");
  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != h->device) return fail(LS_GPU_ERR_INVALID, "sector plan was created on another device");
  for (size_t i = 0; i < h->ops.size(); ++i) {
    auto it = g_ops.find(h->ops[i]);
    if (it == g_ops.end() || it->second != h->caches[i] || !same_terms(it->second->off, h->ops[i]->off_diag_terms) ||
        !same_terms(it->second->diag, h->ops[i]->diag_terms))
      return fail(LS_GPU_ERR_INVALID, "an operator of the sector plan changed after the plan was created");
  }
  return sector_plan_run(h->plan, device_error_word(), (cudaStream_t)stream);
}

extern "C" int ls_gpu_sector_plan_set_batched(void* plan, int batched) {
  SectorPlanHandle* h = (SectorPlanHandle*)plan;
  if (h == nullptr || h->magic != kPlanMagic) return fail(LS_GPU_ERR_INVALID, "not a sector plan");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (sector_plan_set_batched(h->plan, batched != 0) != 0)
    return fail(LS_GPU_ERR_INVALID, "the sectors of this plan cannot share one launch");
  return 0;
}

extern "C" int ls_gpu_sector_plan_autotune(void* plan, void* stream, int* batched, double* ms_batched,
                                           double* ms_per_sector) {
  SectorPlanHandle* h = (SectorPlanHandle*)plan;
  if (h == nullptr || h->magic != kPlanMagic) return fail(LS_GPU_ERR_INVALID, "not a sector plan");
  cudaStream_t s = (cudaStream_t)stream;
  double t[2] = {-1.0, -1.0};  // [per sector, batched]
  bool can_batch = false;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    can_batch = sector_plan_set_batched(h->plan, true) == 0;
  }
  for (int form = can_batch ? 1 : 0; form >= 0; --form) {
    {
      std::lock_guard<std::mutex> lock(g_mutex);
      sector_plan_set_batched(h->plan, form == 1);
    }
    int rc = ls_gpu_sector_plan_run(plan, stream);  // warm-up (uploads, first-touch)
    if (rc != 0) return rc;
    cudaEvent_t e0, e1;
    if (!cuda_ok(cudaEventCreate(&e0), "event") || !cuda_ok(cudaEventCreate(&e1), "event")) return LS_GPU_ERR_CUDA;
    cudaEventRecord(e0, s);
    for (int r = 0; r < 2 && rc == 0; ++r) rc = ls_gpu_sector_plan_run(plan, stream);
    cudaEventRecord(e1, s);
    const bool ok = cuda_ok(cudaEventSynchronize(e1), "autotune sector plan");
    float ms = 0.0f;
    if (ok) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != 0) return rc;
    if (!ok) return LS_GPU_ERR_CUDA;
    t[form] = ms / 2.0;
  }
  const bool use = can_batch && t[1] <= t[0];
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    sector_plan_set_batched(h->plan, use);
  }
  if (batched) *batched = use ? 1 : 0;
  if (ms_batched) *ms_batched = t[1];
  if (ms_per_sector) *ms_per_sector = t[0];
  return 0;
}

extern "C" int ls_gpu_sector_plan_destroy(void* plan) {
  SectorPlanHandle* h = (SectorPlanHandle*)plan;
  if (h == nullptr) return 0;
  if (h->magic != kPlanMagic) return fail(LS_GPU_ERR_INVALID, "not a sector plan");
  std::lock_guard<std::mutex> lock(g_mutex);
  sector_plan_free(h->plan);
  h->magic = 0;
  delete h;
  return 0;
}

extern "C" int ls_gpu_matvec_multi_sector_c128(int n_sectors, ls_hs_operator const* const* ops, int k,
                                               double const* const* d_x, double* const* d_y, int adjoint,
                                               void* stream) {
  void* plan = nullptr;
  int rc = ls_gpu_sector_plan_create(n_sectors, ops, k, d_x, k, d_y, k, adjoint, &plan);
  if (rc != 0) return rc;
  rc = ls_gpu_sector_plan_run(plan, stream);
  if (rc == 0 && !cuda_ok(cudaStreamSynchronize((cudaStream_t)stream), "multi-sector matvec")) rc = LS_GPU_ERR_CUDA;
  const int rc2 = ls_gpu_sector_plan_destroy(plan);
  return rc != 0 ? rc : rc2;
}
