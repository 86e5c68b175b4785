/* CPU restatement of the event-list pair sums -- test infrastructure only.
 *
 * Restates the event correlator of dynamix (resources/opencl/evtcorrelator.cl:3-47,
 * driven by correlator/event.py:162-204): for every pixel p with q-bin b >= 1
 * and events (t_i, v_i), i < n_p, taken from offsets[p] .. offsets[p+1]:
 *     S[b-1][t_i]            += v_i
 *     N[b-1][|t_j - t_i|]    += v_i * v_j      for every pair i <= j.
 * The reference accumulates in 32-bit atomics; this restatement uses int64 so it
 * stays exact on any input.  Threads (POSIX) take pixels from a shared counter
 * and keep private histograms that are summed at the end, so the result does
 * not depend on the thread count.
 *
 * Used by the tests as a checker and by the benchmark as the timed CPU
 * baseline; the product never links it.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  const int32_t* times;
  const void* data;
  int elem_bytes;
  const uint32_t* offsets;
  const int32_t* pix;   /* pixels to process */
  const int32_t* bin;   /* their 0-based bins */
  int64_t n_pix;
  int32_t T;
  int32_t n_bins;
  int64_t* N;           /* [n_bins][T] */
  int64_t* S;
  volatile int64_t next;
  pthread_mutex_t lock;
  int status;
} job_t;

static inline int64_t value_at(const job_t* j, int64_t e) {
  return j->elem_bytes == 1 ? (int64_t)((const uint8_t*)j->data)[e] : (int64_t)((const uint16_t*)j->data)[e];
}

static void* worker(void* arg) {
  job_t* j = (job_t*)arg;
  const size_t cells = (size_t)j->n_bins * (size_t)j->T;
  int64_t* N = (int64_t*)calloc(cells, sizeof(int64_t));
  int64_t* S = (int64_t*)calloc(cells, sizeof(int64_t));
  int bad = 0;
  if (!N || !S) {
    free(N);
    free(S);
    pthread_mutex_lock(&j->lock);
    j->status = 2;
    pthread_mutex_unlock(&j->lock);
    return NULL;
  }
  for (;;) {
    int64_t k = __atomic_fetch_add(&j->next, 64, __ATOMIC_RELAXED);
    if (k >= j->n_pix) break;
    int64_t k1 = k + 64 < j->n_pix ? k + 64 : j->n_pix;
    for (; k < k1; ++k) {
      const int32_t p = j->pix[k];
      const int32_t b = j->bin[k];
      const int64_t o0 = j->offsets[p], o1 = j->offsets[p + 1];
      int64_t* Nb = N + (size_t)b * j->T;
      int64_t* Sb = S + (size_t)b * j->T;
      for (int64_t a = o0; a < o1; ++a) {
        const int32_t ta = j->times[a];
        const int64_t va = value_at(j, a);
        if (ta < 0 || ta >= j->T) {
          bad = 1;
          continue;
        }
        Sb[ta] += va;
        for (int64_t c = a; c < o1; ++c) {
          const int32_t tc = j->times[c];
          if (tc < 0 || tc >= j->T) continue;
          const int32_t lag = tc > ta ? tc - ta : ta - tc;
          Nb[lag] += va * value_at(j, c);
        }
      }
    }
  }
  pthread_mutex_lock(&j->lock);
  for (size_t i = 0; i < cells; ++i) {
    j->N[i] += N[i];
    j->S[i] += S[i];
  }
  if (bad) j->status = 1;
  pthread_mutex_unlock(&j->lock);
  free(N);
  free(S);
  return NULL;
}

/* Pair sums of the listed pixels.  N and S ([n_bins][T] int64) are added to,
 * not cleared.  Returns 0, 1 (an event time outside [0, T)), 2 (out of
 * memory) or 3 (bad argument). */
int g2o_event_pairsum(const int32_t* times, const void* data, int elem_bytes, const uint32_t* offsets,
                      const int32_t* pix, const int32_t* bin, int64_t n_pix, int32_t T, int32_t n_bins,
                      int64_t* N, int64_t* S, int n_threads) {
  if ((elem_bytes != 1 && elem_bytes != 2) || T <= 0 || n_bins <= 0 || n_pix < 0 || n_threads <= 0) return 3;
  for (int64_t k = 0; k < n_pix; ++k)
    if (bin[k] < 0 || bin[k] >= n_bins) return 3;
  job_t j;
  memset(&j, 0, sizeof(j));
  j.times = times;
  j.data = data;
  j.elem_bytes = elem_bytes;
  j.offsets = offsets;
  j.pix = pix;
  j.bin = bin;
  j.n_pix = n_pix;
  j.T = T;
  j.n_bins = n_bins;
  j.N = N;
  j.S = S;
  pthread_mutex_init(&j.lock, NULL);
  if (n_threads > 256) n_threads = 256;
  pthread_t th[256];
  int started = 0;
  for (int i = 0; i < n_threads; ++i)
    if (pthread_create(&th[i], NULL, worker, &j) == 0) ++started;
  if (started == 0) worker(&j);
  for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
  pthread_mutex_destroy(&j.lock);
  return j.status;
}
