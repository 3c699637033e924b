// Batched instances: many independent beams assembled by one persistent
// launch per kernel (no counterpart in the reference, whose Core holds one
// mesh; include/coreimpl.h:11-19).
//
// Each instance is an ordinary context without matrix or state of its own
// (basis tables, geometry cache, law constants, Neumann load, Dirichlet
// rows).  The batch context owns the block-diagonal union: CSR pattern and
// values, state history, residual, Dirichlet rows with instance offsets, so
// Newton, GMRES, SpMV and the CUDA graphs of the single-instance path run on
// it unchanged.
//
// Work queue: every element of every instance, colour-major (colour
// 9*(ex%3) + 3*(ey%3) + ez%3), instances in the schedule's order inside a
// colour.  Persistent CTAs take `grab` items per fetch; an item of colour k
// waits until all its instance's items of colours < k are finished (one
// counter per instance in device memory, bounded waits that set the error
// word).
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace igap {

constexpr int NCOL = 27;
constexpr int HEAD_TC = 32;  // queue heads on separate 128-byte lines

struct Batch {
  int ninst = 0;
  std::vector<Context *> subs;
  std::vector<int64_t> dof_off, elem_off;  // [ninst+1]
  DevMesh *d_mesh = nullptr;
  DevLaw *d_law = nullptr;
  BatchItem *d_items = nullptr;
  int64_t nitems = 0;
  int items_order = -1;    // order the uploaded queue was built with
  int *d_ctrl = nullptr;   // heads [64] | done FP64 kernel [n] | done TC kernel [n]
  int *d_need = nullptr;   // [27n] items of the instance in colours before each colour
  int *d_dir_inst = nullptr;
  int *d_nbs = nullptr;        // [3n]
  int64_t *d_off = nullptr;    // [n+1]
  double *d_norms = nullptr;   // [n]
  igapgpu_batch_schedule sched{1, 1, 1, 0};
  int nsm = 0;
  bool all_geof = false;  // every instance has the FP32 geometry cache
  bool all_gop = false;   // every instance has its cached Gram operands
  int64_t *d_eoff = nullptr;  // [n+1] element offsets (double-FP32 residual)
  float2 *d_rel = nullptr;    // [elements][81] element residual pairs
  int *d_einst = nullptr;     // [elements] instance of each element
  int rdf_state = -1;         // -1 not decided, 0 off, 1 on
  size_t ctrl_bytes() const { return sizeof(int) * (64 + 2 * (size_t)ninst); }
};

template <typename T>
static int balloc(T **p, size_t n)
{
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * n, cudaGetErrorString(e));
    return IGAPGPU_ERR_NOMEM;
  }
  return IGAPGPU_OK;
}

// Colour-major queue and, per (instance, colour), the instance's item count
// in the colours before it.
static int build_items(Context *c, int order)
{
  Batch *b = c->batch;
  if (b->items_order == order && b->d_items) return IGAPGPU_OK;
  const int n = b->ninst;
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  if (order == 1)
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
      return b->subs[x]->nelem_total > b->subs[y]->nelem_total;
    });
  std::vector<BatchItem> items;
  items.reserve((size_t)c->nelem_total);
  std::vector<int> need((size_t)NCOL * n, 0);
  for (int col = 0; col < NCOL; col++) {
    const int cx = col / 9, cy = (col / 3) % 3, cz = col % 3;
    for (int i : ord) {
      const Context *s = b->subs[i];
      for (int ex = cx; ex < s->nelem[0]; ex += 3)
        for (int ey = cy; ey < s->nelem[1]; ey += 3)
          for (int ez = cz; ez < s->nelem[2]; ez += 3) {
            items.push_back(BatchItem{i, col, ex, (ey << 16) | ez});
            need[(size_t)NCOL * i + col]++;
          }
    }
  }
  // exclusive prefix over the colours of each instance: an element of colour
  // k waits for every element of colours < k (empty colours included)
  for (int i = 0; i < n; i++) {
    int run = 0;
    for (int col = 0; col < NCOL; col++) {
      const int cnt = need[(size_t)NCOL * i + col];
      need[(size_t)NCOL * i + col] = run;
      run += cnt;
    }
  }
  b->nitems = (int64_t)items.size();
  if (!b->d_items) {
    int r = balloc(&b->d_items, items.size());
    if (r) return r;
  }
  if (!b->d_need) {
    int r = balloc(&b->d_need, need.size());
    if (r) return r;
  }
  IGAP_CUDA(cudaMemcpy(b->d_items, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice));
  IGAP_CUDA(cudaMemcpy(b->d_need, need.data(), sizeof(int) * need.size(), cudaMemcpyHostToDevice));
  b->items_order = order;
  return IGAPGPU_OK;
}

static BatchArgs batch_args(const Context *c, int which, int64_t nitems)
{
  const Batch *b = c->batch;
  BatchArgs a;
  a.meshes = b->d_mesh;
  a.laws = b->d_law;
  a.items = b->d_items;
  a.nitems = nitems;
  a.head = b->d_ctrl + (which == 0 ? 0 : HEAD_TC);
  a.done = b->d_ctrl + 64 + (size_t)which * b->ninst;
  a.need = b->d_need;
  a.grab = which == 0 ? b->sched.grab_fp64 : b->sched.grab_tc;
  a.err = c->d_err;
  return a;
}

static int fp64_grid(Context *c, bool res, bool tan, int *grid)
{
  int occ = 1;
  int r = element_batch_occupancy(c->law, res, tan, &occ);
  if (r) return r;
  if (occ < 1) occ = 1;
  const int want = c->batch->sched.ctas_per_sm_fp64;
  *grid = c->batch->nsm * (want < occ ? want : occ);
  return IGAPGPU_OK;
}

static int check_err_word(Context *c)
{
  int herr = 0;
  IGAP_CUDA(cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  if (herr == 3) {
    set_error("batched assembly: a bounded wait for a colour of an instance expired");
    return IGAPGPU_ERR_TIMEOUT;
  }
  if (herr) {
    set_error("tensor-core tangent: a bounded mbarrier wait expired (code %d)", herr);
    return IGAPGPU_ERR_TIMEOUT;
  }
  return IGAPGPU_OK;
}

// The linear law's residual in the split mode in double-FP32 arithmetic
// (res_df.cu) when every instance has its FP64 geometry cache and the
// element-residual buffer fits (IGAPGPU_RES_DF=0 keeps the FP64 kernel).
// Decided and allocated once, when the split mode is selected (outside any
// graph capture); the assembly only reads the decision.
static void batch_res_df_setup(Context *c)
{
  Batch *b = c->batch;
  if (b->rdf_state >= 0) return;
  b->rdf_state = 0;
  const char *env = getenv("IGAPGPU_RES_DF");
  bool ok = !(env && env[0] == '0') && c->law == IGAPGPU_LAW_LINGRAD;
  for (Context *s : b->subs) ok = ok && s->d_geo != nullptr;
  if (!ok) return;
  const int64_t nel = b->elem_off[b->ninst];
  std::vector<int> einst((size_t)nel);
  for (int i = 0; i < b->ninst; i++)
    for (int64_t g = b->elem_off[i]; g < b->elem_off[i + 1]; g++) einst[(size_t)g] = i;
  if (cudaMalloc(&b->d_eoff, sizeof(int64_t) * (b->ninst + 1)) == cudaSuccess &&
      cudaMalloc(&b->d_einst, sizeof(int) * (size_t)nel) == cudaSuccess &&
      cudaMalloc(&b->d_rel, sizeof(float2) * NE * (size_t)nel) == cudaSuccess &&
      cudaMemcpy(b->d_eoff, b->elem_off.data(), sizeof(int64_t) * (b->ninst + 1), cudaMemcpyHostToDevice) ==
          cudaSuccess &&
      cudaMemcpy(b->d_einst, einst.data(), sizeof(int) * (size_t)nel, cudaMemcpyHostToDevice) == cudaSuccess) {
    b->rdf_state = 1;
    return;
  }
  cudaGetLastError();
  void *bufs[] = {b->d_eoff, b->d_einst, b->d_rel};
  for (void *p : bufs)
    if (p) cudaFree(p);
  b->d_eoff = nullptr;
  b->d_einst = nullptr;
  b->d_rel = nullptr;
}

static bool batch_res_df(const Context *c)
{
  return c->batch->rdf_state == 1 && c->prec == IGAPGPU_PREC_SPLIT;
}

// The two persistent kernels on the first nitems queue items.
// which: bit 0 = FP64 element kernel (or the residual), bit 1 = tensor-core
// tangent kernel.
static int batch_kernels(Context *c, bool do_res, bool do_tan, double *RR, double *vals, int64_t nitems,
                         int which = 3)
{
  Batch *b = c->batch;
  IGAP_CUDA(cudaMemsetAsync(b->d_ctrl, 0, b->ctrl_bytes(), c->stream));
  IGAP_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
  const bool fp64_tan = do_tan && c->prec != IGAPGPU_PREC_SPLIT;
  // the split mode's residual over every element (nitems: the whole queue)
  if (do_res && nitems == b->nitems && batch_res_df(c)) {
    do_res = false;
    if (which & 1) {
      int r = launch_res_df_batch(c, b->d_mesh, b->d_law, b->d_eoff, b->d_einst, b->d_off, b->ninst,
                                  b->elem_off[b->ninst], b->d_rel, RR);
      if (r) return r;
    }
  }
  if ((do_res || fp64_tan) && (which & 1)) {
    int grid = 0;
    int r = fp64_grid(c, do_res, fp64_tan, &grid);
    if (r) return r;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c->prof) {
      IGAP_CUDA(cudaEventCreate(&e0));
      IGAP_CUDA(cudaEventCreate(&e1));
      IGAP_CUDA(cudaEventRecord(e0, c->stream));
    }
    r = launch_element_batch(c, batch_args(c, 0, nitems), c->law, do_res, fp64_tan, grid, c->d_Uhist, RR,
                             vals);
    if (r) return r;
    if (c->prof) {
      IGAP_CUDA(cudaEventRecord(e1, c->stream));
      c->prof_ev[0].emplace_back(e0, e1);
      c->prof_launches[0]++;
      c->prof_elements[0] += nitems;
    }
  }
  if (do_tan && !fp64_tan && (which & 2)) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c->prof) {
      IGAP_CUDA(cudaEventCreate(&e0));
      IGAP_CUDA(cudaEventCreate(&e1));
      IGAP_CUDA(cudaEventRecord(e0, c->stream));
    }
    int r = (c->law == IGAPGPU_LAW_LINGRAD && b->all_geof && !getenv("IGAPGPU_TC_DENSE"))
                ? launch_tc_gram_batch(c, batch_args(c, 1, nitems), b->nsm, vals, b->all_gop)
                : launch_tc_batch(c, batch_args(c, 1, nitems), c->law, b->nsm, c->d_Uhist, vals);
    if (r) return r;
    if (c->prof) {
      IGAP_CUDA(cudaEventRecord(e1, c->stream));
      c->prof_ev[1].emplace_back(e0, e1);
      c->prof_launches[1]++;
      c->prof_elements[1] += nitems;
    }
  }
  if (!c->capturing) return check_err_word(c);  // a graph replay checks the word itself
  return IGAPGPU_OK;
}

int launch_batch_assembly(Context *c, bool do_res, bool do_tan, double *RR, double *vals)
{
  Batch *b = c->batch;
  if (do_res)
    IGAP_CUDA(cudaMemcpyAsync(RR, c->d_Fneu, sizeof(double) * c->ndof, cudaMemcpyDeviceToDevice, c->stream));
  if (do_tan) IGAP_CUDA(cudaMemsetAsync(vals, 0, sizeof(double) * c->nnz, c->stream));
  int r = batch_kernels(c, do_res, do_tan, RR, vals, b->nitems);
  if (r) return r;
  if (do_res && (r = launch_dirichlet_residual(c, RR))) return r;
  if (do_tan && (r = launch_dirichlet_matrix_batch(c, b->d_dir_inst, b->d_nbs, b->d_off, vals))) return r;
  return IGAPGPU_OK;
}

int batch_set_neumann(Context *c, const double *table)
{
  Batch *b = c->batch;
  for (int i = 0; i < b->ninst; i++) {
    Context *s = b->subs[i];
    for (int k = 0; k < 36; k++) s->bc.neumann[k] = table[k];
    s->stream = c->stream;
    int r = launch_neumann(s, s->nfac);
    if (r) return r;
    IGAP_CUDA(cudaMemcpyAsync(c->d_Fneu + b->dof_off[i], s->d_Fneu, sizeof(double) * s->ndof,
                              cudaMemcpyDeviceToDevice, c->stream));
  }
  for (int k = 0; k < 36; k++) c->bc.neumann[k] = table[k];
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

void batch_release(Context *c)
{
  Batch *b = c->batch;
  if (!b) return;
  for (Context *s : b->subs) context_free(s);
  void *bufs[] = {b->d_mesh, b->d_law, b->d_items, b->d_ctrl, b->d_need, b->d_dir_inst, b->d_nbs, b->d_off,
                  b->d_norms, b->d_eoff, b->d_einst, b->d_rel};
  for (void *p : bufs)
    if (p) cudaFree(p);
  delete b;
  c->batch = nullptr;
}

// Segment norms: one block per instance, fixed reduction tree.
__global__ void __launch_bounds__(256) segment_norm_kernel(const double *__restrict__ x,
                                                           const int64_t *__restrict__ off,
                                                           double *__restrict__ out)
{
  __shared__ double red[8];
  const int i = blockIdx.x;
  const int64_t a = off[i], e = off[i + 1];
  double s = 0.0;
  for (int64_t k = a + threadIdx.x; k < e; k += blockDim.x) s = fma(x[k], x[k], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; w++) t += red[w];
    out[i] = sqrt(t);
  }
}

// Rough device bytes of the batch besides the geometry caches: CSR values and
// columns, state, Krylov basis (restart 100), staging.
// Split precision on a batch: cached Gram operands for every instance (linear
// law); the cached-operand kernel runs only when every instance has them.
int batch_prepare_split(Context *c)
{
  Batch *b = c->batch;
  batch_res_df_setup(c);
  bool all = true;
  for (Context *s : b->subs) {
    const int r = ensure_gram_operands(s);
    if (r) return r;
    all = all && s->d_gop != nullptr;
  }
  b->all_gop = all;
  if (!all) return IGAPGPU_OK;
  std::vector<DevMesh> hm(b->ninst);
  IGAP_CUDA(cudaMemcpy(hm.data(), b->d_mesh, sizeof(DevMesh) * b->ninst, cudaMemcpyDeviceToHost));
  for (int i = 0; i < b->ninst; i++) hm[i].gop = b->subs[i]->d_gop;
  IGAP_CUDA(cudaMemcpy(b->d_mesh, hm.data(), sizeof(DevMesh) * b->ninst, cudaMemcpyHostToDevice));
  return IGAPGPU_OK;
}

static size_t batch_other_bytes(int64_t nnz, int64_t ndof, int torder)
{
  return (size_t)nnz * 12 + (size_t)ndof * 8 * (size_t)(torder + 1 + 8 + 2 * 101);
}

static int64_t instance_nnz(const int nb[3])
{
  auto cnt = [&](int i, int n) { return (i < P ? i : P) + 1 + (i > n - 1 - P ? n - 1 - i : P); };
  int64_t s[3] = {0, 0, 0};
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < nb[d]; i++) s[d] += cnt(i, nb[d]);
  return 9 * s[0] * s[1] * s[2];  // 3 DOF rows x 3 DOF columns per control-point pair
}

}  // namespace igap

using namespace igap;

extern "C" {

int igapgpu_batch_init(igapgpu_t *out, int ninst, const igapgpu_mesh_desc *meshes,
                       const igapgpu_phys_desc *phys, const igapgpu_bc_desc *bcs, int nquad)
{
  if (!out || !meshes || !phys || !bcs || ninst < 1) {
    set_error("batch: null argument or no instance");
    return IGAPGPU_ERR_ARG;
  }
  *out = nullptr;
  for (int i = 0; i < ninst; i++) {
    int r = check_instance_args(meshes + i, phys + i, bcs + i, nquad);
    if (r) return r;
    if (meshes[i].porder != P) {
      set_error("batch: instance %d has degree %d; batches hold quadratic instances", i, meshes[i].porder);
      return IGAPGPU_ERR_ARG;
    }
    if (phys[i].law != phys[0].law) {
      set_error("batch: instance %d has law %d, instance 0 law %d (one law per batch)", i, phys[i].law,
                phys[0].law);
      return IGAPGPU_ERR_ARG;
    }
    if (meshes[i].nelem[1] >= 65536 || meshes[i].nelem[2] >= 65536) {
      set_error("batch: instance %d has more than 65535 elements in y or z", i);
      return IGAPGPU_ERR_ARG;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device: the GPU assembly has no CPU fallback");
    return IGAPGPU_ERR_CUDA;
  }
  Context *c = new_context(meshes, phys, bcs, nquad);
  Batch *b = new Batch();
  c->batch = b;
  b->ninst = ninst;
#define BTRY(x)              \
  do {                       \
    int _r = (x);            \
    if (_r) {                \
      context_free(c);       \
      return _r;             \
    }                        \
  } while (0)
#define BCUDA(x)                                                                             \
  do {                                                                                       \
    cudaError_t _e = (x);                                                                    \
    if (_e != cudaSuccess) {                                                                 \
      set_error("CUDA error %s at %s:%d", cudaGetErrorName(_e), __FILE__, __LINE__);         \
      context_free(c);                                                                       \
      return IGAPGPU_ERR_CUDA;                                                               \
    }                                                                                        \
  } while (0)
  BCUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
  c->stream = c->own_stream;
  int dev = 0;
  BCUDA(cudaGetDevice(&dev));
  BCUDA(cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev));
  // sizes, and the geometry cache mode the free memory allows for all instances
  int64_t ndof = 0, nnz = 0, nel = 0;
  for (int i = 0; i < ninst; i++) {
    const int nb[3] = {meshes[i].nelem[0] + P, meshes[i].nelem[1] + P, meshes[i].nelem[2] + P};
    ndof += 3LL * nb[0] * nb[1] * nb[2];
    nnz += instance_nnz(nb);
    nel += (int64_t)meshes[i].nelem[0] * meshes[i].nelem[1] * meshes[i].nelem[2];
  }
  {
    size_t freeb = 0, totb = 0;
    BCUDA(cudaMemGetInfo(&freeb, &totb));
    const size_t geo = sizeof(double) * (size_t)nel * nquad * nquad * nquad * (NB * NDD + 2);
    const size_t other = batch_other_bytes(nnz, ndof, c->torder) + ((size_t)8 << 30);
    const size_t avail = (size_t)(0.9 * (double)freeb);
    c->geo_mode = (geo + geo / 2 + other < avail) ? 2 : (geo + other < avail ? 1 : 0);
  }
  // instances
  b->dof_off.assign(ninst + 1, 0);
  b->elem_off.assign(ninst + 1, 0);
  for (int i = 0; i < ninst; i++) {
    Context *s = new_context(meshes + i, phys + i, bcs + i, nquad);
    s->sub = true;
    s->stream = c->stream;
    s->geo_mode = c->geo_mode;
    b->subs.push_back(s);
    BTRY(context_init(s, meshes + i));
    b->dof_off[i + 1] = b->dof_off[i] + s->ndof;
    b->elem_off[i + 1] = b->elem_off[i] + s->nelem_total;
  }
  c->ndof = ndof;
  c->ncp = ndof / 3;
  c->nnz = nnz;
  c->nelem_total = nel;
  c->nelem[0] = (int)(nel < 0x7fffffff ? nel : 0x7fffffff);
  c->nelem[1] = c->nelem[2] = 1;
  for (int d = 0; d < 3; d++) c->nbasis[d] = c->nelem[d] + P;
  // block-diagonal CSR
  {
    std::vector<int64_t> rowptr(ndof + 1);
    rowptr[0] = 0;
    int64_t row = 0, base = 0;
    for (int i = 0; i < ninst; i++) {
      const std::vector<int64_t> &rp = b->subs[i]->h_rowptr;
      for (int64_t k = 0; k < b->subs[i]->ndof; k++) rowptr[++row] = base + rp[k + 1];
      base += rp[b->subs[i]->ndof];
    }
    if (base != nnz) {
      set_error("batch: pattern size mismatch (%lld vs %lld)", (long long)base, (long long)nnz);
      context_free(c);
      return IGAPGPU_ERR_ARG;
    }
    if (ndof > INT64_C(2147483647)) {
      set_error("batch: more than 2^31 DOFs");
      context_free(c);
      return IGAPGPU_ERR_ARG;
    }
    BTRY(balloc(&c->d_rowptr, ndof + 1));
    BCUDA(cudaMemcpy(c->d_rowptr, rowptr.data(), sizeof(int64_t) * (ndof + 1), cudaMemcpyHostToDevice));
  }
  BTRY(balloc(&c->d_cols, nnz));
  BTRY(balloc(&c->d_vals, nnz));
  for (int i = 0; i < ninst; i++)
    BTRY(launch_pattern_cols_at(b->subs[i], c->d_rowptr + b->dof_off[i], c->d_cols, b->dof_off[i]));
  // state, residual, staging, reductions
  BTRY(balloc(&c->d_Uhist, (size_t)(c->torder + 1) * ndof));
  BCUDA(cudaMemset(c->d_Uhist, 0, sizeof(double) * (c->torder + 1) * ndof));
  BTRY(balloc(&c->d_RR, ndof));
  BTRY(balloc(&c->d_stage_a, ndof));
  BTRY(balloc(&c->d_stage_b, ndof));
  BTRY(balloc(&c->d_Fneu, ndof));
  BTRY(balloc(&c->d_err, 1));
  BCUDA(cudaMemset(c->d_err, 0, sizeof(int)));
  BTRY(balloc(&c->d_red, 64));
  BTRY(balloc(&c->d_partial, 1024));
  BCUDA(cudaMallocHost(&c->h_red, 64 * sizeof(double)));
  c->red_cap = 64;
  // Neumann load and Dirichlet rows of every instance, with offsets
  std::vector<int64_t> dir_rows;
  std::vector<double> dir_g;
  std::vector<int> dir_inst;
  for (int i = 0; i < ninst; i++) {
    Context *s = b->subs[i];
    BCUDA(cudaMemcpyAsync(c->d_Fneu + b->dof_off[i], s->d_Fneu, sizeof(double) * s->ndof,
                          cudaMemcpyDeviceToDevice, c->stream));
    if (s->n_dir) {
      std::vector<int64_t> rr(s->n_dir);
      std::vector<double> gg(s->n_dir);
      BCUDA(cudaMemcpy(rr.data(), s->d_dir_rows, sizeof(int64_t) * s->n_dir, cudaMemcpyDeviceToHost));
      BCUDA(cudaMemcpy(gg.data(), s->d_dir_g, sizeof(double) * s->n_dir, cudaMemcpyDeviceToHost));
      for (int64_t k = 0; k < s->n_dir; k++) {
        dir_rows.push_back(rr[k] + b->dof_off[i]);
        dir_g.push_back(gg[k]);
        dir_inst.push_back(i);
      }
    }
  }
  c->n_dir = (int64_t)dir_rows.size();
  if (c->n_dir) {
    BTRY(balloc(&c->d_dir_rows, c->n_dir));
    BTRY(balloc(&c->d_dir_g, c->n_dir));
    BTRY(balloc(&b->d_dir_inst, c->n_dir));
    BCUDA(cudaMemcpy(c->d_dir_rows, dir_rows.data(), sizeof(int64_t) * c->n_dir, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(c->d_dir_g, dir_g.data(), sizeof(double) * c->n_dir, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(b->d_dir_inst, dir_inst.data(), sizeof(int) * c->n_dir, cudaMemcpyHostToDevice));
  }
  // per-instance descriptors
  {
    std::vector<DevMesh> hm(ninst);
    std::vector<DevLaw> hl(ninst);
    std::vector<int> nbs(3 * ninst);
    for (int i = 0; i < ninst; i++) {
      Context *s = b->subs[i];
      hm[i] = s->devmesh();
      hm[i].rowptr = c->d_rowptr + b->dof_off[i];
      hm[i].ndof = ndof;
      hm[i].dof_off = b->dof_off[i];
      hl[i] = s->devlaw();
      for (int d = 0; d < 3; d++) nbs[3 * i + d] = s->nbasis[d];
    }
    BTRY(balloc(&b->d_mesh, ninst));
    BTRY(balloc(&b->d_law, ninst));
    BTRY(balloc(&b->d_nbs, 3 * ninst));
    BTRY(balloc(&b->d_off, ninst + 1));
    BTRY(balloc(&b->d_norms, ninst));
    BCUDA(cudaMemcpy(b->d_mesh, hm.data(), sizeof(DevMesh) * ninst, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(b->d_law, hl.data(), sizeof(DevLaw) * ninst, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(b->d_nbs, nbs.data(), sizeof(int) * 3 * ninst, cudaMemcpyHostToDevice));
    BCUDA(cudaMemcpy(b->d_off, b->dof_off.data(), sizeof(int64_t) * (ninst + 1), cudaMemcpyHostToDevice));
  }
  b->all_geof = true;
  for (Context *s : b->subs) b->all_geof = b->all_geof && s->d_geof != nullptr;
  BTRY(balloc(&b->d_ctrl, b->ctrl_bytes() / sizeof(int)));
  BTRY(build_items(c, b->sched.order));
  BCUDA(cudaStreamSynchronize(c->stream));
#undef BTRY
#undef BCUDA
  *out = static_cast<igapgpu_ctx *>(c);
  return IGAPGPU_OK;
}

int igapgpu_batch_info(igapgpu_t c, int *ninst, int64_t *dof_off, int64_t *elem_off)
{
  if (!c || !c->batch) {
    set_error("not a batch context");
    return IGAPGPU_ERR_ARG;
  }
  Batch *b = c->batch;
  if (ninst) *ninst = b->ninst;
  if (dof_off) memcpy(dof_off, b->dof_off.data(), sizeof(int64_t) * (b->ninst + 1));
  if (elem_off) memcpy(elem_off, b->elem_off.data(), sizeof(int64_t) * (b->ninst + 1));
  return IGAPGPU_OK;
}

int igapgpu_batch_norms(igapgpu_t c, const double *x, double *norms)
{
  if (!c || !c->batch || !x || !norms) {
    set_error("batch norms: null argument or not a batch context");
    return IGAPGPU_ERR_ARG;
  }
  Batch *b = c->batch;
  const double *xd = x;
  if (!is_device_ptr(x)) {
    IGAP_CUDA(cudaMemcpyAsync(c->d_stage_a, x, sizeof(double) * c->ndof, cudaMemcpyHostToDevice, c->stream));
    xd = c->d_stage_a;
  }
  segment_norm_kernel<<<b->ninst, 256, 0, c->stream>>>(xd, b->d_off, b->d_norms);
  count_launch();
  IGAP_CHECK_LAUNCH();
  IGAP_CUDA(cudaMemcpyAsync(norms, b->d_norms, sizeof(double) * b->ninst,
                            is_device_ptr(norms) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
  IGAP_CUDA(cudaStreamSynchronize(c->stream));
  return IGAPGPU_OK;
}

int igapgpu_batch_set_schedule(igapgpu_t c, const igapgpu_batch_schedule *s)
{
  if (!c || !c->batch || !s) {
    set_error("batch schedule: null argument or not a batch context");
    return IGAPGPU_ERR_ARG;
  }
  if (s->grab_fp64 < 1 || s->grab_fp64 > 64 || s->grab_tc < 1 || s->grab_tc > 64 || s->ctas_per_sm_fp64 < 1 ||
      s->ctas_per_sm_fp64 > 8 || (s->order != 0 && s->order != 1)) {
    set_error("batch schedule out of range (grab 1..64, ctas_per_sm 1..8, order 0/1)");
    return IGAPGPU_ERR_ARG;
  }
  c->batch->sched = *s;
  int r = build_items(c, s->order);
  if (r) return r;
  graph_release(c);  // captured launches carry the old schedule
  return IGAPGPU_OK;
}

int igapgpu_batch_get_schedule(igapgpu_t c, igapgpu_batch_schedule *s)
{
  if (!c || !c->batch || !s) {
    set_error("batch schedule: null argument or not a batch context");
    return IGAPGPU_ERR_ARG;
  }
  *s = c->batch->sched;
  return IGAPGPU_OK;
}

int igapgpu_batch_autotune(igapgpu_t c, int reps, double frac, igapgpu_batch_schedule *best,
                           double *ms_fp64, double *ms_tc)
{
  if (!c || !c->batch) {
    set_error("autotune: not a batch context");
    return IGAPGPU_ERR_ARG;
  }
  if (reps < 1) reps = 1;
  if (!(frac > 0.0) || frac > 1.0) frac = 1.0;
  Batch *b = c->batch;
  const bool split = c->prec == IGAPGPU_PREC_SPLIT;
  // the FP64 kernel computes the residual (and, in FP64 mode, the tangent)
  const bool tan64 = !split;
  int occ = 1;
  int r = element_batch_occupancy(c->law, true, tan64, &occ);
  if (r) return r;
  if (occ < 1) occ = 1;
  if (occ > 4) occ = 4;
  const int grabs[] = {1, 2, 4, 8};
  cudaEvent_t e0, e1;
  IGAP_CUDA(cudaEventCreate(&e0));
  IGAP_CUDA(cudaEventCreate(&e1));
  const bool prof = c->prof;
  c->prof = false;
  auto time_one = [&](int which, double *ms) -> int {
    const int64_t n = std::max<int64_t>(1, (int64_t)(frac * (double)b->nitems));
    float tmin = 1e30f;
    for (int k = 0; k < reps; k++) {
      IGAP_CUDA(cudaEventRecord(e0, c->stream));
      int rr = batch_kernels(c, which == 1, which == 1 ? tan64 : true, c->d_RR, c->d_vals, n, which);
      if (rr) return rr;
      IGAP_CUDA(cudaEventRecord(e1, c->stream));
      IGAP_CUDA(cudaEventSynchronize(e1));
      float t = 0.f;
      IGAP_CUDA(cudaEventElapsedTime(&t, e0, e1));
      tmin = std::min(tmin, t);
    }
    *ms = tmin;
    return IGAPGPU_OK;
  };
  igapgpu_batch_schedule keep = b->sched, bestS = b->sched;
  double best_total = 1e300, best64 = 0.0, besttc = 0.0;
  for (int order = 0; order < 2 && r == 0; order++) {
    igapgpu_batch_schedule s = b->sched;
    s.order = order;
    if ((r = build_items(c, order))) break;
    double t64 = 1e300, ttc = split ? 1e300 : 0.0;
    int g64 = 1, c64 = 1, gtc = 1;
    for (int g : grabs)
      for (int k = 1; k <= occ && r == 0; k++) {
        b->sched.grab_fp64 = g;
        b->sched.ctas_per_sm_fp64 = k;
        double ms = 0.0;
        if ((r = time_one(1, &ms))) break;
        if (ms < t64) { t64 = ms; g64 = g; c64 = k; }
      }
    if (split)
      for (int g : grabs) {
        if (r) break;
        b->sched.grab_tc = g;
        double ms = 0.0;
        if ((r = time_one(2, &ms))) break;
        if (ms < ttc) { ttc = ms; gtc = g; }
      }
    if (r) break;
    s.grab_fp64 = g64;
    s.ctas_per_sm_fp64 = c64;
    s.grab_tc = gtc;
    if (t64 + ttc < best_total) {
      best_total = t64 + ttc;
      bestS = s;
      best64 = t64;
      besttc = ttc;
    }
    b->sched = keep;
  }
  c->prof = prof;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->matrix_valid = false;
  if (r) {
    b->sched = keep;
    build_items(c, keep.order);
    return r;
  }
  b->sched = bestS;
  if ((r = build_items(c, bestS.order))) return r;
  graph_release(c);
  if (best) *best = bestS;
  if (ms_fp64) *ms_fp64 = best64;
  if (ms_tc) *ms_tc = besttc;
  return IGAPGPU_OK;
}

}  // extern "C"
