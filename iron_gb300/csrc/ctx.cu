// ctx.cu -- handle layer of the C ABI: a context (stream, device error word, mesh cache) and mesh
// handles whose CSR structure and element colouring are built once and shared by every handle of
// the same connectivity.
//
// Iron keeps the equations matrices' structure with the equations set
// (EquationsMatrices_CreateFinish -> EquationsMatrix_StructureCalculate,
// src/equations_matrices_routines.F90:4316-4602) and reuses it for every assembly of that set; a
// gfe_mesh plays that role here.  The context owns what Iron's per-rank globals hold: the error
// state (one device error word per context, so contexts on different host threads do not see
// each other's kernel errors) and the structures, cached by a hash of the connectivity so that
// several equations sets on one mesh share them.
#include <algorithm>
#include <climits>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "gfe_internal.cuh"

struct gfe_mesh_cache_entry {
  int device = 0;
  int32_t n_elem = 0, n_nodes = 0, npe = 0;
  int32_t nx = 0, ny = 0, nz = 0;  // > 0: Iron's regular generated mesh of nx x ny x nz elements
  std::vector<int32_t> host_nodes;  // connectivity (to resolve hash collisions)
  int32_t* elem_nodes = nullptr;    // device copy
  int32_t* row_ptr = nullptr;
  int32_t* col_idx = nullptr;
  int64_t nnz = 0;
  int32_t* color_elems = nullptr;
  std::vector<int32_t> color_ptr;
  bool regular_ok = false;  // structure verified as the clipped 27-point stencil
  ~gfe_mesh_cache_entry() {
    int cur = 0;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != device) cudaSetDevice(device);
    cudaFree(elem_nodes);
    cudaFree(row_ptr);
    cudaFree(col_idx);
    cudaFree(color_elems);
    if (cur != device) cudaSetDevice(cur);
  }
};

struct gfe_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  unsigned* err = nullptr;
  std::mutex mu;
  std::map<uint64_t, std::vector<std::shared_ptr<gfe_mesh_cache_entry>>> cache;
};

struct gfe_mesh {
  gfe_ctx* ctx = nullptr;
  std::shared_ptr<gfe_mesh_cache_entry> entry;
};

namespace {

// FNV-1a over the connectivity and its sizes
uint64_t fnv1a(const void* data, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

// Routes the kernels of the calling thread to the context's error word for the life of the guard.
struct ErrorWordScope {
  unsigned* prev;
  explicit ErrorWordScope(unsigned* w) : prev(gfe::thread_error_word()) { gfe::set_thread_error_word(w); }
  ~ErrorWordScope() { gfe::set_thread_error_word(prev); }
};

int check_ctx(gfe_ctx* ctx, const char* fn) {
  if (!ctx) return gfe::set_error(GFE_ERR_ARG, "%s: context is NULL", fn);
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != ctx->device)
    return gfe::set_error(GFE_ERR_ARG, "%s: the context belongs to device %d, the current device is %d", fn,
                          ctx->device, dev);
  return GFE_OK;
}

// Greedy element colouring in element order: each element takes the lowest colour that none of
// its nodes' earlier elements has (at most 64 colours).
int greedy_colours(const std::vector<int32_t>& en, int32_t n_elem, int32_t npe, int32_t n_nodes,
                   std::vector<int32_t>& order, std::vector<int32_t>& ptr) {
  std::vector<uint64_t> used(n_nodes, 0ull);
  std::vector<int8_t> colour(n_elem);
  int ncol = 0;
  for (int32_t e = 0; e < n_elem; ++e) {
    uint64_t u = 0;
    for (int32_t k = 0; k < npe; ++k) u |= used[en[(size_t)e * npe + k]];
    if (u == ~0ull) return gfe::set_error(GFE_ERR_ARG, "gfe_mesh_create: more than 64 element colours needed");
    int c = 0;
    while (u & (1ull << c)) ++c;
    colour[e] = (int8_t)c;
    ncol = std::max(ncol, c + 1);
    for (int32_t k = 0; k < npe; ++k) used[en[(size_t)e * npe + k]] |= 1ull << c;
  }
  ptr.assign(ncol + 1, 0);
  for (int32_t e = 0; e < n_elem; ++e) ++ptr[colour[e] + 1];
  for (int c = 0; c < ncol; ++c) ptr[c + 1] += ptr[c];
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  order.assign(n_elem, 0);
  for (int32_t e = 0; e < n_elem; ++e) order[fill[colour[e]]++] = e;
  return GFE_OK;
}

// parity colouring of a regular mesh: colour = (e1 & 1) + 2 (e2 & 1) + 4 (e3 & 1), element order kept
void parity_colours(int32_t nx, int32_t ny, int32_t nz, std::vector<int32_t>& order, std::vector<int32_t>& ptr) {
  const int32_t E = nx * ny * nz;
  ptr.assign(9, 0);
  auto col = [&](int32_t e) { return (e % nx & 1) + 2 * ((e / nx) % ny & 1) + 4 * (e / (nx * ny) & 1); };
  for (int32_t e = 0; e < E; ++e) ++ptr[col(e) + 1];
  for (int c = 0; c < 8; ++c) ptr[c + 1] += ptr[c];
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  order.assign(E, 0);
  for (int32_t e = 0; e < E; ++e) order[fill[col(e)]++] = e;
}

int build_entry(gfe_ctx* ctx, gfe_mesh_cache_entry& m, const char* fn) {
  cudaStream_t s = ctx->stream;
  const size_t conn = (size_t)m.n_elem * m.npe;
  GFE_CUDA_TRY(cudaMalloc(&m.elem_nodes, std::max<size_t>(conn, 1) * sizeof(int32_t)));
  GFE_CUDA_TRY(cudaMemcpyAsync(m.elem_nodes, m.host_nodes.data(), conn * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  GFE_CUDA_TRY(cudaMalloc(&m.row_ptr, ((size_t)m.n_nodes + 1) * sizeof(int32_t)));
  int64_t nnz = 0;
  int rc = gfe_csr_structure(m.n_elem, m.npe, m.elem_nodes, m.n_nodes, m.row_ptr, nullptr, 0, &nnz, s);
  if (rc) return rc;
  GFE_CUDA_TRY(cudaMalloc(&m.col_idx, std::max<int64_t>(nnz, 1) * sizeof(int32_t)));
  if ((rc = gfe_csr_structure(m.n_elem, m.npe, m.elem_nodes, m.n_nodes, m.row_ptr, m.col_idx, nnz, &nnz, s)))
    return rc;
  m.nnz = nnz;
  std::vector<int32_t> order;
  if (m.nx > 0) {
    parity_colours(m.nx, m.ny, m.nz, order, m.color_ptr);
    int64_t bad = -1;
    if ((rc = gfe_laplace_regular_check(m.nx, m.ny, m.nz, m.row_ptr, m.col_idx, &bad, s))) return rc;
    m.regular_ok = bad == 0;
  } else if ((rc = greedy_colours(m.host_nodes, m.n_elem, m.npe, m.n_nodes, order, m.color_ptr))) {
    return rc;
  }
  GFE_CUDA_TRY(cudaMalloc(&m.color_elems, std::max<size_t>(order.size(), 1) * sizeof(int32_t)));
  GFE_CUDA_TRY(cudaMemcpyAsync(m.color_elems, order.data(), order.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  GFE_CUDA_TRY(cudaStreamSynchronize(s));
  (void)fn;
  return GFE_OK;
}

int lookup_or_build(gfe_ctx* ctx, std::shared_ptr<gfe_mesh_cache_entry> cand, gfe_mesh** out, const char* fn) {
  uint64_t h = fnv1a(&cand->n_nodes, sizeof(int32_t));
  h = fnv1a(&cand->npe, sizeof(int32_t), h);
  h = fnv1a(&cand->nx, 3 * sizeof(int32_t), h);
  h = fnv1a(cand->host_nodes.data(), cand->host_nodes.size() * sizeof(int32_t), h);
  std::lock_guard<std::mutex> lk(ctx->mu);
  for (auto& e : ctx->cache[h]) {
    if (e->n_elem == cand->n_elem && e->n_nodes == cand->n_nodes && e->npe == cand->npe && e->nx == cand->nx &&
        e->ny == cand->ny && e->nz == cand->nz && e->host_nodes == cand->host_nodes) {
      *out = new gfe_mesh{ctx, e};
      return GFE_OK;
    }
  }
  cand->device = ctx->device;
  int rc = build_entry(ctx, *cand, fn);
  if (rc) return rc;
  ctx->cache[h].push_back(cand);
  *out = new gfe_mesh{ctx, cand};
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_ctx_create(void* stream, gfe_ctx** out) {
  if (!out) return gfe::set_error(GFE_ERR_ARG, "gfe_ctx_create: out is NULL");
  *out = nullptr;
  auto* c = new gfe_ctx;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaMalloc(&c->err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(c->err, 0, sizeof(unsigned));
  if (e != cudaSuccess) {
    cudaFree(c->err);
    delete c;
    return gfe::set_error(GFE_ERR_CUDA, "gfe_ctx_create: %s", cudaGetErrorString(e));
  }
  c->stream = gfe::as_stream(stream);
  *out = c;
  return GFE_OK;
}

extern "C" int gfe_ctx_destroy(gfe_ctx* ctx) {
  if (!ctx) return GFE_OK;
  cudaStreamSynchronize(ctx->stream);
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->cache.clear();  // entries still held by live mesh handles are freed with the last handle
  }
  cudaFree(ctx->err);
  delete ctx;
  return GFE_OK;
}

extern "C" int gfe_ctx_device_errors(gfe_ctx* ctx, uint32_t* bits_host) {
  const char* fn = "gfe_ctx_device_errors";
  int rc = check_ctx(ctx, fn);
  if (rc) return rc;
  if (!bits_host) return gfe::set_error(GFE_ERR_ARG, "%s: bits_host is NULL", fn);
  unsigned v = 0;
  GFE_CUDA_TRY(cudaMemcpyAsync(&v, ctx->err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  GFE_CUDA_TRY(cudaMemsetAsync(ctx->err, 0, sizeof(unsigned), ctx->stream));
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  *bits_host = v;
  return GFE_OK;
}

extern "C" int gfe_ctx_cached_meshes(gfe_ctx* ctx, int32_t* count_host) {
  const char* fn = "gfe_ctx_cached_meshes";
  if (!ctx || !count_host) return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  std::lock_guard<std::mutex> lk(ctx->mu);
  int32_t n = 0;
  for (auto& kv : ctx->cache) n += (int32_t)kv.second.size();
  *count_host = n;
  return GFE_OK;
}

extern "C" int gfe_mesh_create(gfe_ctx* ctx, int32_t n_elem, int32_t nodes_per_elem, const int32_t* elem_nodes_host,
                               int32_t n_nodes, gfe_mesh** out) {
  const char* fn = "gfe_mesh_create";
  int rc = check_ctx(ctx, fn);
  if (rc) return rc;
  if (!out || n_elem <= 0 || nodes_per_elem <= 0 || n_nodes <= 0 || !elem_nodes_host)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  *out = nullptr;
  auto cand = std::make_shared<gfe_mesh_cache_entry>();
  cand->n_elem = n_elem;
  cand->npe = nodes_per_elem;
  cand->n_nodes = n_nodes;
  cand->host_nodes.assign(elem_nodes_host, elem_nodes_host + (size_t)n_elem * nodes_per_elem);
  for (int32_t v : cand->host_nodes)
    if (v < 0 || v >= n_nodes) return gfe::set_error(GFE_ERR_ARG, "%s: node number %d outside [0, %d)", fn, v, n_nodes);
  return lookup_or_build(ctx, cand, out, fn);
}

extern "C" int gfe_mesh_create_regular(gfe_ctx* ctx, int32_t nx, int32_t ny, int32_t nz, gfe_mesh** out) {
  const char* fn = "gfe_mesh_create_regular";
  int rc = check_ctx(ctx, fn);
  if (rc) return rc;
  if (!out || nx <= 0 || ny <= 0 || nz <= 0 || (int64_t)(nx + 1) * (ny + 1) * (nz + 1) > INT32_MAX)
    return gfe::set_error(GFE_ERR_ARG, "%s: invalid arguments", fn);
  *out = nullptr;
  auto cand = std::make_shared<gfe_mesh_cache_entry>();
  cand->nx = nx;
  cand->ny = ny;
  cand->nz = nz;
  cand->npe = 8;
  cand->n_elem = nx * ny * nz;
  const int32_t NX = nx + 1, NY = ny + 1;
  cand->n_nodes = NX * NY * (nz + 1);
  // Iron's regular generated mesh (src/generated_mesh_routines.F90:1568-1640): elements and
  // nodes xi1 fastest, local nodes xi1 fastest
  cand->host_nodes.resize((size_t)cand->n_elem * 8);
  for (int32_t k = 0; k < nz; ++k)
    for (int32_t j = 0; j < ny; ++j)
      for (int32_t i = 0; i < nx; ++i) {
        const size_t e = (size_t)i + (size_t)j * nx + (size_t)k * nx * ny;
        const int32_t first = i + j * NX + k * NX * NY;
        for (int m = 0; m < 8; ++m)
          cand->host_nodes[e * 8 + m] = first + (m & 1) + ((m >> 1) & 1) * NX + (m >> 2) * NX * NY;
      }
  return lookup_or_build(ctx, cand, out, fn);
}

extern "C" int gfe_mesh_destroy(gfe_mesh* mesh) {
  delete mesh;
  return GFE_OK;
}

extern "C" int gfe_mesh_csr(const gfe_mesh* mesh, const int32_t** row_ptr, const int32_t** col_idx, int64_t* nnz,
                            int32_t* n_rows) {
  if (!mesh) return gfe::set_error(GFE_ERR_ARG, "gfe_mesh_csr: mesh is NULL");
  if (row_ptr) *row_ptr = mesh->entry->row_ptr;
  if (col_idx) *col_idx = mesh->entry->col_idx;
  if (nnz) *nnz = mesh->entry->nnz;
  if (n_rows) *n_rows = mesh->entry->n_nodes;
  return GFE_OK;
}

extern "C" int gfe_assemble_laplace(gfe_ctx* ctx, const gfe_mesh* mesh, const double* coords, const double* kappa_e,
                                    double* values, float* values32, double* rhs, int32_t precision) {
  const char* fn = "gfe_assemble_laplace";
  int rc = check_ctx(ctx, fn);
  if (rc) return rc;
  if (!mesh || mesh->ctx != ctx) return gfe::set_error(GFE_ERR_ARG, "%s: mesh does not belong to this context", fn);
  if (!coords || !values) return gfe::set_error(GFE_ERR_ARG, "%s: coords and values are required", fn);
  const gfe_mesh_cache_entry& m = *mesh->entry;
  if (m.npe != 8)
    return gfe::set_error(GFE_ERR_ARG, "%s: the mesh has %d nodes per element; trilinear hexahedra have 8", fn, m.npe);
  ErrorWordScope scope(ctx->err);
  // FP64 element arithmetic is bound by the FP64 pipe, where the colour kernel (each element once)
  // beats the tiled kernel (halo elements recomputed); the FP32-pipe precisions take the tiled
  // row-owning kernel on Iron's regular generated mesh
  if (m.nx > 0 && m.regular_ok && precision != GFE_FP64)
    return gfe_laplace_assemble_regular(m.nx, m.ny, m.nz, coords, kappa_e, m.row_ptr, values, values32, rhs,
                                        precision, ctx->stream);
  return gfe_laplace_assemble(m.n_elem, m.n_nodes, m.elem_nodes, coords, kappa_e, m.color_elems, m.color_ptr.data(),
                              (int32_t)m.color_ptr.size() - 1, m.row_ptr, m.col_idx, m.nnz, values, values32, rhs,
                              precision, ctx->stream);
}

extern "C" int gfe_solve_laplace(gfe_ctx* ctx, const gfe_mesh* mesh, const double* values, const float* values32,
                                 const double* f, const uint8_t* fixed, double* x, double rtol, int32_t max_iters,
                                 int32_t precision, int32_t* iters_host, double* rel_host) {
  const char* fn = "gfe_solve_laplace";
  int rc = check_ctx(ctx, fn);
  if (rc) return rc;
  if (!mesh || mesh->ctx != ctx) return gfe::set_error(GFE_ERR_ARG, "%s: mesh does not belong to this context", fn);
  const gfe_mesh_cache_entry& m = *mesh->entry;
  ErrorWordScope scope(ctx->err);
  return gfe_cg_solve(m.n_nodes, m.row_ptr, m.col_idx, values, values32, f, fixed, x, rtol, max_iters, precision,
                      iters_host, rel_host, ctx->stream);
}
