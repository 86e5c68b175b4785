/* Host driver that runs the reference's event kernels (compiled as C through
 * opencl_shim.h) over their NDRanges -- test infrastructure only.
 *
 * g2r_event_correlate follows EventCorrelator.correlate (dynamix
 * correlator/event.py:162-204): event_correlator over the (W, H) grid, then
 * normalize_correlation over (nframes, n_bins).  The caller passes the scalar
 * arguments exactly as the reference does, including its image_height
 * argument (event.py:183 passes shape[1]).  Work-items run on n_threads POSIX
 * threads, rows split among them; the kernels' atomics are real atomics.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>

#include "opencl_shim.h"

_Thread_local size_t g2r_gid[3];
int g2r_image_width;
int g2r_num_bins;

/* the kernels, as compiled from the reference's file (DTYPE erased to void) */
void event_correlator(const int* vol_times_array, const void* vol_data_array, const uint* offsets,
                      const int* q_mask, int* res_tau, uint* sums, int image_height, int Nt);
void normalize_correlation(int* res_int, float* res, uint* sums, float* scale_factors, int Nt);

typedef struct {
  const int* times;
  const void* data;
  const uint* offsets;
  const int* qmask;
  int* res_int;
  uint* sums;
  int image_height_arg;
  int Nt;
  size_t grid_w, grid_h;
  size_t row0, row1;
} ev_slice;

static void* ev_worker(void* arg) {
  ev_slice* s = (ev_slice*)arg;
  for (size_t y = s->row0; y < s->row1; ++y)
    for (size_t x = 0; x < s->grid_w; ++x) {
      g2r_gid[0] = x;
      g2r_gid[1] = y;
      g2r_gid[2] = 0;
      event_correlator(s->times, s->data, s->offsets, s->qmask, s->res_int, s->sums, s->image_height_arg, s->Nt);
    }
  return NULL;
}

/* MAX_EVT_COUNT of the compiled kernel file */
int g2r_max_evt_count(void) { return MAX_EVT_COUNT; }

/* Returns 0, or 3 when an argument is out of range (the caller checks that no
 * pixel has more than g2r_max_evt_count() events: the kernel does not). */
int g2r_event_correlate(const int32_t* times, const void* data, const uint32_t* offsets, const int32_t* qmask,
                        int32_t* res_int, uint32_t* sums, float* res, float* scale_factors, int width,
                        int height, int image_height_arg, int nframes, int n_bins, int n_threads) {
  if (width <= 0 || height <= 0 || nframes <= 0 || n_bins <= 0 || n_threads <= 0) return 3;
  g2r_image_width = width;
  g2r_num_bins = n_bins;
  if (n_threads > 64) n_threads = 64;
  if ((size_t)n_threads > (size_t)height) n_threads = height;
  ev_slice sl[64];
  pthread_t th[64];
  int started[64] = {0};
  for (int i = 0; i < n_threads; ++i) {
    ev_slice s = {times, data, offsets, qmask, res_int, sums, image_height_arg, nframes,
                  (size_t)width, (size_t)height, (size_t)height * i / n_threads,
                  (size_t)height * (i + 1) / n_threads};
    sl[i] = s;
    started[i] = pthread_create(&th[i], NULL, ev_worker, &sl[i]) == 0;
    if (!started[i]) ev_worker(&sl[i]);
  }
  for (int i = 0; i < n_threads; ++i)
    if (started[i]) pthread_join(th[i], NULL);
  for (int b = 0; b < n_bins; ++b)
    for (int t = 0; t < nframes; ++t) {
      g2r_gid[0] = (size_t)t;
      g2r_gid[1] = (size_t)b;
      normalize_correlation(res_int, res, sums, scale_factors, nframes);
    }
  return 0;
}
