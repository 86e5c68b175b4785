/* Host driver that runs the reference's dense and CSR OpenCL kernels
 * (compiled as C through opencl_wg_shim.h) over their NDRanges -- test
 * infrastructure only.
 *
 * One work-group runs at a time; its work-items are POSIX threads that stay
 * alive for the whole launch and walk the groups together.  Built with
 * -DG2W_DENSE (densecorrelator.cl: correlator_multiQ_dense, compute_sums_dense,
 * correlate_1D, launched as DenseCorrelator.correlate does,
 * dynamix/correlator/dense.py:170-272) or -DG2W_CSR (correlator.cl:
 * compute_sums, correlator_oneQ_Nt, launched as SparseCorrelator.correlate
 * does, dynamix/correlator/intensity.py:80-129).  Each g2w_* entry point
 * returns 0, or 3 for an argument it cannot launch.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

#include "opencl_wg_shim.h"

_Thread_local size_t g2w_lid[3];
_Thread_local size_t g2w_grp[3];
size_t g2w_lsize[3];

/* ---- the barrier over the live threads of the running group ------------- */
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t g_cv = PTHREAD_COND_INITIALIZER;
static size_t g_live, g_arrived, g_generation;
static pthread_barrier_t g_group_end;

void g2w_barrier(void) {
  pthread_mutex_lock(&g_mu);
  const size_t gen = g_generation;
  if (++g_arrived >= g_live) {
    g_arrived = 0;
    ++g_generation;
    pthread_cond_broadcast(&g_cv);
  } else {
    while (gen == g_generation) pthread_cond_wait(&g_cv, &g_mu);
  }
  pthread_mutex_unlock(&g_mu);
}

/* a thread leaves the kernel body: it no longer holds up a barrier */
static void leave_body(void) {
  pthread_mutex_lock(&g_mu);
  --g_live;
  if (g_arrived > 0 && g_arrived >= g_live) {
    g_arrived = 0;
    ++g_generation;
    pthread_cond_broadcast(&g_cv);
  }
  pthread_mutex_unlock(&g_mu);
}

typedef void (*body_fn)(void* ctx);
typedef struct {
  size_t lid, ngroups0, ngroups1;
  body_fn body;
  void* ctx;
} worker_arg;

static void* worker(void* p) {
  worker_arg* w = (worker_arg*)p;
  g2w_lid[0] = w->lid;
  g2w_lid[1] = g2w_lid[2] = 0;
  for (size_t g1 = 0; g1 < w->ngroups1; ++g1)
    for (size_t g0 = 0; g0 < w->ngroups0; ++g0) {
      g2w_grp[0] = g0;
      g2w_grp[1] = g1;
      g2w_grp[2] = 0;
      w->body(w->ctx);
      leave_body();
      pthread_barrier_wait(&g_group_end);   /* every thread is out of this group */
      if (w->lid == 0) {
        g_live = g2w_lsize[0];
        g_arrived = 0;
      }
      pthread_barrier_wait(&g_group_end);   /* the next group starts with all threads live */
    }
  return NULL;
}

/* Run a 2-D NDRange (global gsize0 x gsize1, local lsize0 x 1). */
static int run_ndrange(size_t gsize0, size_t gsize1, size_t lsize0, body_fn body, void* ctx) {
  if (lsize0 == 0 || lsize0 > 1024 || gsize0 % lsize0 != 0 || gsize1 == 0) return 3;
  g2w_lsize[0] = lsize0;
  g2w_lsize[1] = g2w_lsize[2] = 1;
  g_live = lsize0;
  g_arrived = 0;
  if (pthread_barrier_init(&g_group_end, NULL, (unsigned)lsize0) != 0) return 3;
  pthread_t* th = (pthread_t*)calloc(lsize0, sizeof(pthread_t));
  worker_arg* args = (worker_arg*)calloc(lsize0, sizeof(worker_arg));
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, 1 << 18);
  int rc = 0;
  size_t started = 0;
  for (size_t i = 0; i < lsize0; ++i) {
    worker_arg a = {i, gsize0 / lsize0, gsize1, body, ctx};
    args[i] = a;
    if (pthread_create(&th[i], &attr, worker, &args[i]) != 0) {
      rc = 3;
      break;
    }
    ++started;
  }
  if (rc != 0) abort();   /* a partial group would wait forever: fail loudly */
  for (size_t i = 0; i < started; ++i) pthread_join(th[i], NULL);
  pthread_attr_destroy(&attr);
  pthread_barrier_destroy(&g_group_end);
  free(th);
  free(args);
  return rc;
}

#ifdef G2W_DENSE
/* the kernels, as compiled from the reference's densecorrelator.cl */
void correlator_multiQ_dense(const char* frames, const int* q_mask, const float* normalization, float* output,
                             int image_height, int Nt);
void compute_sums_dense(const void* frames, const int* q_mask, uint* sums, int image_height, int Nt);
void correlate_1D(const uint* sums, float* output);

typedef struct {
  const void* frames;
  const int* qmask;
  const float* norm;
  float* out_f;
  uint* sums;
  int image_height, nt;
} dense_ctx;

static void body_numerator(void* p) {
  dense_ctx* c = (dense_ctx*)p;
  correlator_multiQ_dense((const char*)c->frames, c->qmask, c->norm, c->out_f, c->image_height, c->nt);
}
static void body_sums(void* p) {
  dense_ctx* c = (dense_ctx*)p;
  compute_sums_dense(c->frames, c->qmask, c->sums, c->image_height, c->nt);
}
static void body_corr1d(void* p) {
  dense_ctx* c = (dense_ctx*)p;
  correlate_1D(c->sums, c->out_f);
}

/* compute_sums_dense over (SUM_WG_SIZE, Nt) with work-groups (SUM_WG_SIZE, 1)
 * (dense.py:247-258: the launch uses wg[0] = SUM_WG_SIZE). */
int g2w_dense_sums(const void* frames, const int32_t* qmask, uint32_t* sums, int image_height, int nt) {
  dense_ctx c = {frames, qmask, NULL, NULL, sums, image_height, nt};
  return run_ndrange(SUM_WG_SIZE, (size_t)nt, SUM_WG_SIZE, body_sums, &c);
}

/* correlate_1D over (Nt, n_bins) (dense.py:261-271: no work-group size). */
int g2w_dense_corr1d(const uint32_t* sums, float* out, int nt, int n_bins) {
  dense_ctx c = {NULL, NULL, NULL, out, (uint*)sums, 0, nt};
  return run_ndrange((size_t)nt, (size_t)n_bins, 1, body_corr1d, &c);
}

/* correlator_multiQ_dense over (max(wg0, W), Nt) with work-groups (wg0, 1)
 * (dense.py:185-190, 224-235). */
int g2w_dense_numerator(const int8_t* frames, const int32_t* qmask, const float* norm, float* out,
                        int image_height, int nt, int wg0) {
  dense_ctx c = {frames, qmask, norm, out, NULL, image_height, nt};
  const size_t g0 = (size_t)(wg0 > IMAGE_WIDTH ? wg0 : IMAGE_WIDTH);
  return run_ndrange(g0, (size_t)nt, (size_t)wg0, body_numerator, &c);
}
#endif

#ifdef G2W_CSR
/* the kernels, as compiled from the reference's correlator.cl (IDX_DTYPE int) */
void compute_sums(const void* data, const int* offsets, float* output, int Nt);
void correlator_oneQ_Nt(const void* data, const int* indices, const int* indptr, const int* offsets,
                        const float* norm_mask, const float* images_sums, float* output, int image_height,
                        int Nt);

typedef struct {
  const void* data;
  const int *indices, *indptr, *offsets;
  const float *norm_mask, *images_sums;
  float* out;
  int image_height, nt;
} csr_ctx;

static void body_csr_sums(void* p) {
  csr_ctx* c = (csr_ctx*)p;
  compute_sums(c->data, c->offsets, c->out, c->nt);
}
static void body_csr_corr(void* p) {
  csr_ctx* c = (csr_ctx*)p;
  correlator_oneQ_Nt(c->data, c->indices, c->indptr, c->offsets, c->norm_mask, c->images_sums, c->out,
                     c->image_height, c->nt);
}

/* compute_sums over (1024, Nt), work-groups (1024, 1) (intensity.py:92-102). */
int g2w_csr_sums(const void* data, const int32_t* offsets, float* out, int nt) {
  csr_ctx c = {data, NULL, NULL, offsets, NULL, NULL, out, 0, nt};
  return run_ndrange(1024, (size_t)nt, 1024, body_csr_sums, &c);
}

/* correlator_oneQ_Nt over (64, Nt), work-groups (64, 1) (intensity.py:113-126). */
int g2w_csr_correlate(const void* data, const int32_t* indices, const int32_t* indptr, const int32_t* offsets,
                      const float* norm_mask, const float* images_sums, float* out, int image_height, int nt) {
  csr_ctx c = {data, indices, indptr, offsets, norm_mask, images_sums, out, image_height, nt};
  return run_ndrange(64, (size_t)nt, 64, body_csr_corr, &c);
}
#endif
