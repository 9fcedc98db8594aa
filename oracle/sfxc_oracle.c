/*
 * sfxc_oracle.c -- CPU restatement of the SFXC correlator-node hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against (tests/, __graft_entry__.smoke and bench.py's CPU baseline); the
 * product never links, imports or runs it.  Parity is pinned: the
 * tests compare this program's outputs with the reference's own classes run
 * on the same jobs (oracle/ref_harness.cc, fixtures in tests/golden/).
 *
 * Every stage restates the reference's algorithm step by step; each function
 * cites the reference file:line it follows (paths relative to the reference
 * project).  Two arithmetic modes:
 *   precision 32  -- the reference's own arithmetic: float buffers, float
 *                    products and accumulation, double phases (default);
 *   precision 64  -- the same algorithm carried in double throughout, used
 *                    as the FP64 yardstick for error statements.
 * FFTs are computed in double (split into a half-length complex FFT for real
 * input) and, in precision 32, rounded to float like FFTW's float plans.
 *
 * Command line (same job files and output files as oracle/ref_harness.cc):
 *   sfxc_oracle correlate|delays|protocol|extract <job> <out>
 */
#define _GNU_SOURCE
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t ticks_t;
#define CLOCK_RATE 512000000.0 /* MAX_SAMPLE_RATE, sfxc/include/utils.h:36 */
#define REFERENCE_MJD 51544
#define SECONDS_PER_DAY 86400
#define HEADER_DATA 0 /* sfxc/include/utils.h:39-42 */
#define HEADER_INVALID 1
#define HEADER_DELAY 2
#define HEADER_ENDSTREAM 3
#define CORRELATOR_BUFFER_SIZE 8192 /* sfxc/include/utils.h:50 */
#define WINDOW_NONE 0 /* sfxc/include/utils.h (window ids) */
#define WINDOW_RECT 1
#define WINDOW_COS 2
#define WINDOW_HAMMING 3
#define WINDOW_HANN 4

static int g_f64 = 0; /* precision 64 mode */

static void die(const char *m) {
  fprintf(stderr, "sfxc_oracle: %s\n", m);
  exit(2);
}
static void *xmalloc(size_t n) {
  void *p = calloc(1, n ? n : 1);
  if (!p) die("out of memory");
  return p;
}
static void *xrealloc(void *p, size_t n) {
  p = realloc(p, n ? n : 1);
  if (!p) die("out of memory");
  return p;
}
/* storage rounding: float in precision 32, identity in precision 64 */
static inline double st(double x) { return g_f64 ? x : (double)(float)x; }

/* byte vector */
typedef struct {
  unsigned char *p;
  size_t n, cap;
} bytes_t;
static void bpush(bytes_t *b, const void *src, size_t n) {
  if (b->n + n > b->cap) {
    b->cap = (b->n + n) * 2 + 64;
    b->p = xrealloc(b->p, b->cap);
  }
  memcpy(b->p + b->n, src, n);
  b->n += n;
}

/* ------------------------------------------------------------------ time ---
 * Time (sfxc/include/correlator_time.h:58-91, sfxc/src/correlator_time.cc) */
static const ticks_t TICKS_PER_DAY = (ticks_t)SECONDS_PER_DAY * 512000000LL;
static ticks_t t_from_mjd_sec(int mjd, double sec) { /* Time::set_time */
  return (ticks_t)((mjd - REFERENCE_MJD) * SECONDS_PER_DAY * CLOCK_RATE) + (ticks_t)round(sec * CLOCK_RATE);
}
static ticks_t t_from_usec(double usec) { return (ticks_t)round(usec * (CLOCK_RATE / 1000000)); }
static int t_sample_rate(double sr) { return (int)round(CLOCK_RATE / sr); }
static double t_get_mjd(ticks_t t) { /* correlator_time.cc:217-222 */
  int ndays = (int)(t / TICKS_PER_DAY);
  double mjd = REFERENCE_MJD + ndays;
  return mjd + (t % TICKS_PER_DAY) / CLOCK_RATE / SECONDS_PER_DAY;
}
static double t_get_time_usec(ticks_t t) { return (t % TICKS_PER_DAY) / (CLOCK_RATE / 1000000); }
static double t_get_time(ticks_t t) { return (t % TICKS_PER_DAY) / CLOCK_RATE; }
static double t_diff(ticks_t a, ticks_t b) { return (a - b) / CLOCK_RATE; }
static ticks_t t_mul(ticks_t t, double v) { return (ticks_t)round(t * v); }
static ticks_t t_div(ticks_t t, double v) { return (ticks_t)round(t / v); }

/* ------------------------------------------------------------ delay table ---
 * Delay_table::open (sfxc/src/delay_table_akima.cc:238-372) for single-source
 * scans, create_akima_spline (431-502), Delay_table_akima::delay/rate/phase/
 * amplitude (114-166).  The spline is GSL 1.9's Akima (interpolation/akima.c:
 * akima_init + akima_calc, non-periodic boundary; evaluation in Horner form). */
typedef struct {
  ticks_t begin, end;
  int times, vals; /* first row index */
} scan_t;
typedef struct {
  scan_t *scans;
  int nscans;
  double *times, *delays, *phases, *amps;
  int nrows;
  double clock_offset, clock_rate;
  ticks_t clock_epoch;
} deltable_t;

typedef struct {
  int n;
  double *x, *y[3], *b[3], *c[3], *d[3]; /* y: delay, phase, amplitude */
  ticks_t scan_begin, interval_begin, interval_end, clock_epoch;
  double clock_offset, clock_rate;
} akima_t;

static void deltable_read(deltable_t *t, const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) die("cannot open delay table");
  int32_t hs;
  if (fread(&hs, 4, 1, f) != 1) die("bad delay table");
  if (fseek(f, hs, SEEK_CUR)) die("bad delay table");
  memset(t, 0, sizeof(*t));
  int cap = 1024;
  t->times = xmalloc(cap * 8);
  t->delays = xmalloc(cap * 8);
  t->phases = xmalloc(cap * 8);
  t->amps = xmalloc(cap * 8);
  char src[81];
  int32_t mjd;
  double line[7];
  while (fread(src, 1, 81, f) == 81) {
    if (fread(&mjd, 4, 1, f) != 1 || fread(line, 8, 7, f) != 7) break;
    double scan_start = line[0], scan_end = line[0];
    t->scans = xrealloc(t->scans, (t->nscans + 1) * sizeof(scan_t));
    scan_t *s = &t->scans[t->nscans++];
    s->begin = t_from_mjd_sec(mjd, scan_start);
    s->times = s->vals = t->nrows;
    /* an additional phase centre of the same scan is a scan with the same
       start (delay_table_akima.cc:330-336): its rows repeat the times */
    for (;;) {
      if (line[0] == 0 && line[4] == 0) {
        if (t->nrows - s->times == 1) die("delay table scan with a single row");
        s->end = t_from_mjd_sec(mjd, scan_end);
        break;
      }
      if (t->nrows == cap) {
        cap *= 2;
        t->times = xrealloc(t->times, cap * 8);
        t->delays = xrealloc(t->delays, cap * 8);
        t->phases = xrealloc(t->phases, cap * 8);
        t->amps = xrealloc(t->amps, cap * 8);
      }
      t->times[t->nrows] = line[0] - scan_start;
      t->delays[t->nrows] = line[4];
      t->phases[t->nrows] = line[5];
      t->amps[t->nrows] = line[6];
      t->nrows++;
      scan_end = line[0];
      if (fread(line, 8, 7, f) != 7) break;
    }
  }
  fclose(f);
  if (t->nscans == 0) die("empty delay table");
}

/* akima_init / akima_calc, GSL 1.9 interpolation/akima.c:93-154 */
static void akima_coeffs(const double *x, const double *y, int size, double *b, double *c, double *d) {
  double *mbuf = xmalloc((size + 4) * sizeof(double));
  double *m = mbuf + 2;
  for (int i = 0; i <= size - 2; i++) m[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
  m[-2] = 3.0 * m[0] - 2.0 * m[1];
  m[-1] = 2.0 * m[0] - m[1];
  m[size - 1] = 2.0 * m[size - 2] - m[size - 3];
  m[size] = 3.0 * m[size - 2] - 2.0 * m[size - 3];
  for (int i = 0; i < size - 1; i++) {
    const double NE = fabs(m[i + 1] - m[i]) + fabs(m[i - 1] - m[i - 2]);
    if (NE == 0.0) {
      b[i] = m[i];
      c[i] = 0.0;
      d[i] = 0.0;
    } else {
      const double h_i = x[i + 1] - x[i];
      const double NE_next = fabs(m[i + 2] - m[i + 1]) + fabs(m[i] - m[i - 1]);
      const double alpha_i = fabs(m[i - 1] - m[i - 2]) / NE;
      double tL_ip1;
      if (NE_next == 0.0) {
        tL_ip1 = m[i];
      } else {
        const double alpha_ip1 = fabs(m[i] - m[i - 1]) / NE_next;
        tL_ip1 = (1.0 - alpha_ip1) * m[i] + alpha_ip1 * m[i + 1];
      }
      b[i] = (1.0 - alpha_i) * m[i - 1] + alpha_i * m[i];
      c[i] = (3.0 * m[i] - 2.0 * b[i] - tL_ip1) / h_i;
      d[i] = (b[i] + tL_ip1 - 2.0 * m[i]) / (h_i * h_i);
    }
  }
  free(mbuf);
}

/* Delay_table::create_akima_spline (delay_table_akima.cc:431-502); phase
   centre pc: the pc-th scan starting with the covering one (an additional
   phase centre is a scan with the same start, 313-336, 478-494) */
static void akima_create_pc(akima_t *a, const deltable_t *t, ticks_t start_, ticks_t duration, int pc);
static void akima_create(akima_t *a, const deltable_t *t, ticks_t start_, ticks_t duration) {
  akima_create_pc(a, t, start_, duration, 0);
}
static void akima_create_pc(akima_t *a, const deltable_t *t, ticks_t start_, ticks_t duration, int pc) {
  int mjd_start = (int)floor(t_get_mjd(start_));
  double seconds_start = floor(t_get_time_usec(start_) / 1000000);
  ticks_t stop = start_ + duration;
  int mjd_stop = (int)floor(t_get_mjd(stop));
  double seconds_stop = ceil(t_get_time_usec(stop) / 1000000);
  ticks_t start = t_from_mjd_sec(mjd_start, seconds_start);
  int n_seconds = (int)((mjd_stop - mjd_start) * 86400 + seconds_stop - seconds_start);
  int sn = 0;
  while (sn < t->nscans && stop > t->scans[sn].end) sn++;
  if (sn == t->nscans) die("time is not in the delay table");
  if (sn + pc >= t->nscans || t->scans[sn + pc].begin != t->scans[sn].begin)
    die("delay table has fewer phase centres than requested");
  const scan_t *s = &t->scans[sn + pc];
  if (t_diff(s->end, s->begin) < 4.) die("delay table scan shorter than 4 s");
  ticks_t onesec = t_from_usec(1000000.);
  ticks_t ib = start - t_mul(onesec, 2);
  ticks_t ie = start + t_mul(onesec, 2 + n_seconds);
  if (ib < s->begin) {
    ib = s->begin;
    if (t_diff(ie, ib) < 4) ie = ib + t_mul(onesec, 4);
  }
  if (ie > s->end) {
    ie = s->end;
    if (t_diff(ie, ib) < 4) ib = ie - t_mul(onesec, 4);
  }
  int n_pts = (int)((double)(ie - ib) / onesec + 1);
  int idx = (int)t_diff(ib, s->begin);
  if (n_pts <= 4) die("fewer than 5 spline points");
  memset(a, 0, sizeof(*a));
  a->n = n_pts;
  a->x = t->times + s->times + idx;
  const double *cols[3] = {t->delays, t->phases, t->amps};
  for (int k = 0; k < 3; k++) {
    a->y[k] = (double *)cols[k] + s->vals + idx;
    a->b[k] = xmalloc(n_pts * 8);
    a->c[k] = xmalloc(n_pts * 8);
    a->d[k] = xmalloc(n_pts * 8);
    akima_coeffs(a->x, a->y[k], n_pts, a->b[k], a->c[k], a->d[k]);
  }
  a->scan_begin = s->begin;
  a->interval_begin = ib;
  a->interval_end = ie;
  a->clock_epoch = t->clock_epoch;
  a->clock_offset = t->clock_offset;
  a->clock_rate = t->clock_rate;
}
static void akima_free(akima_t *a) {
  for (int k = 0; k < 3; k++) {
    free(a->b[k]);
    free(a->c[k]);
    free(a->d[k]);
  }
}
/* Interval lookup: gsl_interp_bsearch (GSL interpolation/bsearch.c).  GSL's
   accelerator can keep the left interval when x equals a node exactly; the two
   choices agree to rounding (the spline is continuous). */
static int akima_index(const akima_t *a, double x) {
  if (x < a->x[0] || x > a->x[a->n - 1]) die("spline evaluated outside its interval");
  size_t ilo = 0, ihi = a->n - 1;
  while (ihi > ilo + 1) {
    size_t i = (ihi + ilo) / 2;
    if (a->x[i] > x)
      ihi = i;
    else
      ilo = i;
  }
  return (int)ilo;
}
static double akima_eval(const akima_t *a, int k, double x) { /* akima_eval */
  int i = akima_index(a, x);
  const double delx = x - a->x[i];
  return a->y[k][i] + delx * (a->b[k][i] + delx * (a->c[k][i] + a->d[k][i] * delx));
}
static double akima_deriv(const akima_t *a, int k, double x) { /* akima_eval_deriv */
  int i = akima_index(a, x);
  double delx = x - a->x[i];
  return a->b[k][i] + delx * (2.0 * a->c[k][i] + 3.0 * a->d[k][i] * delx);
}
static double dt_delay(const akima_t *a, ticks_t t) { /* delay_table_akima.cc:114-126 */
  if (t < a->interval_begin || t > a->interval_end) die("delay requested outside the spline interval");
  double sec = t_diff(t, a->scan_begin);
  double result = akima_eval(a, 0, sec);
  sec = t_diff(t, a->clock_epoch);
  double clock_drift = a->clock_offset + sec * a->clock_rate;
  return result + clock_drift;
}
static double dt_rate(const akima_t *a, ticks_t t) {
  double sec = t_diff(t, a->scan_begin);
  return akima_deriv(a, 0, sec) + a->clock_rate;
}
static double dt_phase(const akima_t *a, ticks_t t) { return akima_eval(a, 1, t_diff(t, a->scan_begin)); }
static double dt_amplitude(const akima_t *a, ticks_t t) { return akima_eval(a, 2, t_diff(t, a->scan_begin)); }

/* ---------------------------------------------------------- integer delays ---
 * Input_node_tasklet::get_delay / get_delays (sfxc/src/input_node_tasklet.cc:235-282) */
typedef struct {
  ticks_t time;
  int32_t bytes, rem;
} delay_t;
typedef struct {
  delay_t *v;
  int n, cap;
} dlist_t;
static void dl_push(dlist_t *l, delay_t d) {
  if (l->n == l->cap) {
    l->cap = l->cap * 2 + 16;
    l->v = xrealloc(l->v, l->cap * sizeof(delay_t));
  }
  l->v[l->n++] = d;
}
static delay_t get_delay(const akima_t *a, ticks_t time, int sample_rate, int bps) {
  double delay_ = dt_delay(a, time);
  int32_t dis = (int32_t)floor(delay_ * sample_rate + .5);
  int32_t bytes = (int)floor((dis - 1) * 1. / (8 / bps));
  int32_t rem = dis - bytes * (8 / bps);
  if (rem * bps == 8) {
    bytes++;
    rem = 0;
  }
  delay_t d = {time, bytes, rem};
  return d;
}
static void get_delays(const akima_t *a, ticks_t start, int64_t nsamples, int tps, int sr, int bps,
                       dlist_t *out) {
  ticks_t stop = start + nsamples * tps;
  if (!(stop > start)) die("empty delay interval");
  delay_t ds = get_delay(a, start, sr, bps), de = get_delay(a, stop, sr, bps);
  if (de.bytes != ds.bytes || de.rem != ds.rem) {
    if (nsamples == 1) {
      dl_push(out, de);
    } else {
      get_delays(a, start, nsamples / 2, tps, sr, bps, out);
      get_delays(a, start + (nsamples / 2) * tps, nsamples - nsamples / 2, tps, sr, bps, out);
    }
  } else {
    int rate_different = (dt_rate(a, start) * dt_rate(a, stop)) < 0;
    if (rate_different && nsamples >= 3) {
      get_delays(a, start, nsamples / 2, tps, sr, bps, out);
      get_delays(a, start + (nsamples / 2) * tps, nsamples - nsamples / 2, tps, sr, bps, out);
    }
  }
}
/* Input_node_tasklet::add_time_interval (input_node_tasklet.cc:103-115) */
static void interval_delays(const akima_t *a, ticks_t start, ticks_t stop, int sr, int bps, dlist_t *out) {
  int tps = t_sample_rate(sr);
  dl_push(out, get_delay(a, start, sr, bps));
  int64_t nsamples = (stop - start) / tps;
  get_delays(a, start, nsamples, tps, sr, bps, out);
}

/* ---------------------------------------------------------- protocol writer ---
 * Input_node_data_writer (sfxc/src/input_node_data_writer.cc:107-229, 389-500) */
typedef struct {
  int begin, n;
} inval_t;
typedef struct {
  ticks_t start;
  const unsigned char *data;
  int size;
  inval_t *inv;
  int ninv;
} cblock_t;
typedef struct {
  ticks_t start, stop;
  int64_t nr_samples;
  dlist_t delays;
} pslice_t;

static void pw_delay(bytes_t *o, int8_t d) {
  unsigned char h[2] = {HEADER_DELAY, (unsigned char)d};
  bpush(o, h, 2);
}
static void pw_invalid(bytes_t *o, int n) {
  int w = 0;
  while (w < n) {
    int16_t k = (int16_t)((n - w) < SHRT_MAX ? (n - w) : SHRT_MAX);
    unsigned char h = HEADER_INVALID;
    bpush(o, &h, 1);
    bpush(o, &k, 2);
    w += k;
  }
}
static void pw_data(bytes_t *o, const unsigned char *blk, int n, int off) {
  if (n == 0) return;
  int w = 0, start = off;
  while (w < n) {
    int16_t k = (int16_t)((n - w) < SHRT_MAX ? (n - w) : SHRT_MAX);
    unsigned char h = HEADER_DATA;
    bpush(o, &h, 1);
    bpush(o, &k, 2);
    bpush(o, blk + start, k);
    w += k;
    start += k;
  }
}

/* ---------------------------------------------------------- phase cal ---
 * Input_node_data_writer::do_phasecal (sfxc/src/input_node_data_writer.cc:
 * 230-312): the samples of every block the writer takes up, folded modulo
 * sample_rate / 10 kHz into int32 bins; a block starting on a multiple of the
 * phase-cal integration time sends the bins so far (after the first such
 * block) and starts again.  The per-byte loop checks one invalid run per
 * byte, as written. */
typedef struct {
  int64_t T; /* integration ticks, 0: off */
  int sr, bps, P;
  int32_t *acc;
  int64_t count;
  ticks_t time;
  unsigned char station, freq, sb, pol;
  bytes_t out;
  int done; /* blocks processed (input_element.processed) */
} pcal_t;
static void pcal_block(pcal_t *pc, const cblock_t *b, int index) {
  static const int8_t v2[] = {-7, -2, 2, 7}, v1[] = {-5, 5};
  if (!pc || pc->T == 0 || index < pc->done) return;
  pc->done = index + 1;
  const int spb = 8 / pc->bps;
  if (b->start % pc->T == 0) {
    if (pc->P == 0) {
      pc->P = (int)(pc->sr / 10e3);
      pc->acc = xmalloc(pc->P * sizeof(int32_t));
    } else {
      int64_t t0 = pc->time, dt = b->start - pc->time;
      int32_t ns = pc->P;
      bpush(&pc->out, &pc->station, 1);
      bpush(&pc->out, &pc->freq, 1);
      bpush(&pc->out, &pc->sb, 1);
      bpush(&pc->out, &pc->pol, 1);
      bpush(&pc->out, &t0, 8);
      bpush(&pc->out, &dt, 8);
      bpush(&pc->out, &ns, 4);
      bpush(&pc->out, pc->acc, (size_t)pc->P * 4);
      memset(pc->acc, 0, pc->P * sizeof(int32_t));
    }
    pc->count = 0;
    pc->time = b->start;
    if (pc->P % spb) die("phase-cal bins not a whole number of bytes");
  }
  if (pc->P == 0) return;
  int iv = 0;
  for (int i = 0; i < b->size; i++) {
    if (iv < b->ninv && i == b->inv[iv].begin) {
      i += b->inv[iv].n;
      pc->count += (int64_t)b->inv[iv].n * spb;
      iv++;
      if (i >= b->size) break;
    }
    pc->count %= pc->P;
    for (int q = 0; q < spb; q++)
      pc->acc[pc->count++] += pc->bps == 2 ? v2[(b->data[i] >> (2 * q)) & 3] : v1[(b->data[i] >> q) & 1];
  }
}

/* Returns per-slice protocol buffers (and feeds pc, if given, as do_task does). */
static void protocol_write(const cblock_t *blocks, int nblocks, pslice_t *slices, int nslices, int sr,
                           int bps, double integr_time_us, bytes_t *outs, pcal_t *pcal) {
  const int tps = t_sample_rate(sr);
  const ticks_t byte_length = t_from_usec(8 * 1000000. / ((double)sr * bps));
  const ticks_t integration_time = t_from_usec(integr_time_us);
  const int spb = 8 / bps;
  ticks_t current_time = 0, slice_start = 0;
  ticks_t iv_stop = 0;
  int next_interval = 0, writer = 0, active = 0, sync_stream = 0, delay_index = 0;
  int64_t slice_size = nslices ? slices[0].nr_samples : 0;
  const dlist_t *cur = NULL;
  int bi = 0;
  int block_size = 0;
  long guard = 0;
  for (;;) {
    if (++guard > 200000000L) die("protocol writer did not terminate");
    /* has_work (input_node_data_writer.cc:70-103) */
    if (writer >= nslices) break;
    if (!active && current_time >= iv_stop) {
      if (next_interval >= nslices) break;
      /* fetch_next_time_interval (376-386) */
      iv_stop = slices[next_interval].stop;
      delay_index = 0;
      cur = &slices[next_interval].delays;
      current_time = slices[next_interval].start;
      next_interval++;
    }
    if (bi >= nblocks) break;
    /* do_task */
    const cblock_t *blk = &blocks[bi];
    pcal_block(pcal, blk, bi);
    bytes_t *o = &outs[writer];
    int64_t byte_offset = 0;
    int delay_size = cur->n;
    if (!active) {
      active = 1;
      slice_start = current_time;
      sync_stream = 1;
    }
    if (sync_stream) {
      block_size = blk->size;
      while (delay_index < delay_size - 1 && cur->v[delay_index + 1].time <= current_time + byte_length)
        delay_index++;
      int64_t dsamples = (current_time - blk->start) / tps;
      byte_offset = dsamples * bps / 8 + cur->v[delay_index].bytes;
      if (byte_offset < 0) {
        /* write_initial_invalid_data (464-500) */
        int initial_delay = cur->v[delay_index].rem;
        pw_delay(o, (int8_t)cur->v[delay_index].rem);
        slice_size += cur->v[delay_index].rem;
        int64_t invalid_samples = (-byte_offset * spb < slice_size) ? -byte_offset * spb : slice_size;
        int64_t written = 0;
        while (written < invalid_samples) {
          int64_t next_delay_pos;
          if (delay_index < delay_size - 1) {
            ticks_t dt = cur->v[delay_index + 1].time - current_time;
            next_delay_pos = (int64_t)(spb * ((double)dt / byte_length));
          } else {
            next_delay_pos = slice_size * 2;
          }
          if (written == next_delay_pos) {
            delay_index++;
            pw_delay(o, (int8_t)cur->v[delay_index].rem);
            int d = cur->v[delay_index].rem - cur->v[delay_index - 1].rem;
            if (d > 1 || d == -1)
              slice_size -= 1;
            else
              slice_size += 1;
            invalid_samples = (-byte_offset * spb < slice_size) ? -byte_offset * spb : slice_size;
          } else {
            int64_t a1 = next_delay_pos - written, a2 = invalid_samples - written;
            int data_to_write = (int)(a1 < a2 ? a1 : a2);
            pw_invalid(o, data_to_write);
            written += data_to_write;
          }
        }
        slice_size -= invalid_samples;
        current_time += (invalid_samples - initial_delay) * tps;
        sync_stream = 0;
        continue;
      } else if (byte_offset >= block_size) {
        bi++;
        continue;
      } else {
        slice_size += cur->v[delay_index].rem;
        pw_delay(o, (int8_t)cur->v[delay_index].rem);
        current_time -= (ticks_t)cur->v[delay_index].rem * tps;
        sync_stream = 0;
      }
    }
    int index = (int)byte_offset;
    int invalid_index = 0;
    int next_invalid_pos = blk->ninv > 0 ? blk->inv[0].begin : block_size + 1;
#define NEXT_DELAY_POS()                                                             \
  ((delay_index < delay_size - 1)                                                   \
       ? (int)((double)(cur->v[delay_index + 1].time - current_time) / byte_length) \
       : INT_MAX / 2)
    int ndp = NEXT_DELAY_POS();
    int next_delay_pos = (ndp > 0 ? ndp : 0) + (int)byte_offset;
    int64_t tt = (slice_size + spb - 1) / spb;
    int total_to_write = (int)((block_size - byte_offset) < tt ? (block_size - byte_offset) : tt);
    int end_index = total_to_write + (int)byte_offset;
    while (index < end_index) {
      if (index >= next_delay_pos) {
        delay_index++;
        pw_delay(o, (int8_t)cur->v[delay_index].rem);
        int d = cur->v[delay_index].rem - cur->v[delay_index - 1].rem;
        if (d > 1 || d == -1)
          slice_size -= 1;
        else
          slice_size += 1;
        ndp = NEXT_DELAY_POS();
        next_delay_pos = (ndp > 0 ? ndp : 0) + (int)byte_offset;
        tt = (slice_size + spb - 1) / spb;
        total_to_write = (int)((block_size - byte_offset) < tt ? (block_size - byte_offset) : tt);
        end_index = total_to_write + (int)byte_offset;
      } else if (index >= next_invalid_pos) {
        int n = blk->inv[invalid_index].n;
        int end_pos = (next_invalid_pos + n < next_delay_pos) ? next_invalid_pos + n : next_delay_pos;
        int nr_invalid = end_pos - index > 0 ? end_pos - index : 0;
        if (end_index - index < nr_invalid) nr_invalid = end_index - index;
        if (nr_invalid > 0) {
          pw_invalid(o, nr_invalid * spb);
          index += nr_invalid;
        }
        if (end_pos == next_invalid_pos + n) {
          invalid_index++;
          next_invalid_pos = blk->ninv > invalid_index ? blk->inv[invalid_index].begin : block_size + 1;
        }
      } else {
        int dw = next_delay_pos - index < end_index - index ? next_delay_pos - index : end_index - index;
        if (next_invalid_pos - index < dw) dw = next_invalid_pos - index;
        pw_data(o, blk->data, dw, index);
        index += dw;
      }
    }
#undef NEXT_DELAY_POS
    slice_size -= (int64_t)total_to_write * spb;
    current_time += (ticks_t)total_to_write * spb * tps;
    if (index >= block_size) bi++;
    if (slice_size <= 0) {
      unsigned char h = HEADER_ENDSTREAM;
      bpush(o, &h, 1);
      current_time = slice_start + integration_time;
      active = 0;
      writer++;
      if (writer < nslices) slice_size = slices[writer].nr_samples;
    }
  }
}

/* ------------------------------------------------------------------- FFT ---
 * Double-precision radix-2 FFT; real transforms through a half-length complex
 * transform.  Conventions of FFTW (sfxc/src/sfxc_fft_float.cc:103-243):
 * unnormalised, forward sign -1, backward +1, r2c gives n/2+1 bins. */
typedef struct {
  int n;
  double *wr, *wi; /* exp(-2 pi i k / n) */
  int *rev;
} fftplan_t;
static fftplan_t *fft_plan(int n) {
  if (n < 2 || (n & (n - 1))) die("FFT sizes must be powers of two");
  fftplan_t *p = xmalloc(sizeof(*p));
  p->n = n;
  p->wr = xmalloc(n * 8);
  p->wi = xmalloc(n * 8);
  p->rev = xmalloc(n * sizeof(int));
  for (int k = 0; k < n; k++) {
    double a = -2.0 * M_PI * (double)k / (double)n;
    p->wr[k] = cos(a);
    p->wi[k] = sin(a);
  }
  int lg = 0;
  while ((1 << lg) < n) lg++;
  for (int i = 0; i < n; i++) {
    int r = 0;
    for (int b = 0; b < lg; b++)
      if (i & (1 << b)) r |= 1 << (lg - 1 - b);
    p->rev[i] = r;
  }
  return p;
}
/* in-place complex FFT of interleaved re/im, sign -1 (forward) or +1 */
static void fft_c(const fftplan_t *p, double *re, double *im, int sign) {
  const int n = p->n;
  for (int i = 0; i < n; i++) {
    int j = p->rev[i];
    if (i < j) {
      double t = re[i];
      re[i] = re[j];
      re[j] = t;
      t = im[i];
      im[i] = im[j];
      im[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int step = n / len, h = len / 2;
    for (int i = 0; i < n; i += len) {
      for (int j = 0; j < h; j++) {
        double wr = p->wr[j * step], wi = sign < 0 ? p->wi[j * step] : -p->wi[j * step];
        double xr = re[i + j + h], xi = im[i + j + h];
        double vr = xr * wr - xi * wi, vi = xr * wi + xi * wr;
        re[i + j + h] = re[i + j] - vr;
        im[i + j + h] = im[i + j] - vi;
        re[i + j] += vr;
        im[i + j] += vi;
      }
    }
  }
}
/* r2c of n real values through one n/2-point complex FFT; out has n/2+1 bins.
   ph = plan(n/2), pn = plan(n) for the split twiddles. */
static void fft_r2c(const fftplan_t *ph, const fftplan_t *pn, const double *x, double *ore, double *oim,
                    double *wre, double *wim) {
  const int h = ph->n;
  for (int k = 0; k < h; k++) {
    wre[k] = x[2 * k];
    wim[k] = x[2 * k + 1];
  }
  fft_c(ph, wre, wim, -1);
  for (int k = 0; k <= h; k++) {
    int k1 = k % h, k2 = (h - k) % h;
    double er = 0.5 * (wre[k1] + wre[k2]), ei = 0.5 * (wim[k1] - wim[k2]);
    double orr = 0.5 * (wim[k1] + wim[k2]), oi = -0.5 * (wre[k1] - wre[k2]);
    double c = pn->wr[k % pn->n], s = pn->wi[k % pn->n];
    if (k == h) { c = -1.0; s = 0.0; }
    ore[k] = er + (orr * c - oi * s);
    oim[k] = ei + (orr * s + oi * c);
  }
}

/* ----------------------------------------------------------- job structure */
typedef struct {
  int station_number, station_stream, sample_rate, bandwidth, bps, tsys_freq, table;
  int64_t channel_freq;
  char sideband, pol;
  double LO_offset;
} stream_t;

typedef struct {
  ticks_t experiment_start, start;
  double integration_time_us, sub_integration_time_us;
  int number_channels, Nd, M, sample_rate, bandwidth, frequency_nr, cross_polarize, reference_station,
      window, integration_nr, n_integrations;
  int64_t channel_freq;
  char sideband, pol;
  int nstreams;
  stream_t *streams;
  int pulsar, nbins;
  double gate0, gate1;
  int npolyco;
  double *polyco; /* per polyco: tmid DM ref_phase ref_freq obs_freq ncoef coef... (packed, stride 32) */
  int dump;
  int dump_bins; /* the pulsar bin table only */
  /* spectral reduction (number_channels < fft_size_correlation): the
     Mask_parameters of the ctrl file -- a mask over the M+1 channels, a lag
     window over 2 number_channels lags, and the per-channel normalisation;
     NULL / 0 when absent (mask of ones, window from the window type) */
  double *mask, *lag_window;
  /* u, v, w per integration, stream and phase centre for the timeslice
   * headers (NULL: zeros), as Correlator_node::set_parameters hands them to
   * the core (sfxc/src/correlator_node.cc:327-357) */
  double *uvw;
  size_t n_uvw;
  int mask_normalize;
  /* phase centres (Correlation_parameters::n_phase_centers) and the output
     file index of each (the manager's source list; 0 when absent) */
  int n_pc;
  int *pc_file;
  int phased; /* Correlation_core_phased (the phased-array core) */
} job_t;

/* ------------------------------------------------------------- statistics ---
 * bit_statistics (sfxc/src/bit_statistics.cc:22-139) */
typedef struct {
  int64_t on[256], off[256];
  int64_t ninvalid;
  int bps, sr, base_sr;
} bstat_t;
static void stats_levels(const bstat_t *s, int out[5]) { /* get_statistics */
  int64_t st5[5] = {0, 0, 0, 0, 0};
  if (s->bps == 2) {
    for (int i = 0; i < 256; i++) {
      int64_t c = s->on[i] + s->off[i];
      st5[i & 3] += c;
      st5[(i >> 2) & 3] += c;
      st5[(i >> 4) & 3] += c;
      st5[(i >> 6) & 3] += c;
    }
  } else {
    for (int i = 0; i < 256; i++)
      for (int j = 0; j < 8; j++) st5[(i >> j) & 1] += s->on[i] + s->off[i];
  }
  st5[4] += s->ninvalid;
  for (int i = 0; i < 5; i++) {
    int v = (int)st5[i]; /* the reference accumulates in int */
    out[i] = (int)(((uint64_t)s->base_sr * (uint64_t)(int64_t)v) / (uint64_t)s->sr);
  }
}
static void stats_tsys(const bstat_t *s, int out[4]) { /* get_tsys */
  int64_t on[4] = {0}, off[4] = {0};
  out[0] = out[1] = out[2] = out[3] = 0;
  if (s->bps != 2) return;
  for (int i = 0; i < 256; i++) {
    for (int k = 0; k < 4; k++) {
      on[(i >> (2 * k)) & 3] += s->on[i];
      off[(i >> (2 * k)) & 3] += s->off[i];
    }
  }
  out[0] = (int)(on[1] + on[2]);
  out[1] = (int)(on[0] + on[3]);
  out[2] = (int)(off[1] + off[2]);
  out[3] = (int)(off[0] + off[3]);
}

/* --------------------------------------------------------------- bit2float ---
 * Bit2float_worker (sfxc/src/bit2float_worker.cc:36-197, 278-313, 327-436).
 * Restated as a single pass over one integration's protocol with all input
 * available; produces the float stream, the invalid list and the byte
 * histograms exactly as the reference's buffer-by-buffer state machine does. */
enum { B_IDLE, B_SEND_INVALID, B_SEND_DATA, B_PURGE };
static const float SAMPLE_MS[4] = {-7, -2, 2, 7};
static const float SAMPLE_M[2] = {-5, 5};

typedef struct {
  /* persistent across integrations */
  int state;
  size_t bytes_left, invalid_left, sample_in_byte;
  int8_t cur_delay;
  /* per integration */
  int n_ffts, nfft_max, fft_size, bps, sr, base_sr, tsys_freq;
  int tsys_count, tsys_on;
  bstat_t stats;
  inval_t *inv;
  int ninv, capinv;
} b2f_t;

static void b2f_set_parameters(b2f_t *w, const job_t *j, const stream_t *s, double delay_at_start) {
  /* set_new_parameters (237-276) + set_parameters (278-313) */
  int Nd = j->Nd, M = j->M;
  int nfft_min = M / Nd > 1 ? M / Nd : 1;
  int a = CORRELATOR_BUFFER_SIZE / Nd > nfft_min ? CORRELATOR_BUFFER_SIZE / Nd : nfft_min;
  w->nfft_max = (int)(((uint64_t)a * (uint64_t)s->sample_rate) / j->sample_rate);
  ticks_t tint = t_from_usec(j->integration_time_us);
  int nr;
  if (M > Nd) {
    ticks_t tf = t_from_usec(M / (j->sample_rate / 1000000.));
    nr = (int)floor((double)tint / tf);
    w->n_ffts = (int)(((uint64_t)(M / Nd) * nr * (uint64_t)s->sample_rate) / j->sample_rate);
  } else {
    ticks_t tf = t_from_usec(Nd / (j->sample_rate / 1000000.));
    nr = (int)floor((double)tint / tf);
    w->n_ffts = (int)(((uint64_t)nr * (uint64_t)s->sample_rate) / j->sample_rate);
  }
  w->fft_size = Nd;
  w->bps = s->bps;
  w->sr = s->sample_rate;
  w->base_sr = j->sample_rate;
  w->tsys_freq = s->tsys_freq;
  memset(&w->stats, 0, sizeof(w->stats));
  w->stats.bps = s->bps;
  w->stats.sr = s->sample_rate;
  w->stats.base_sr = j->sample_rate;
  w->invalid_left = 0;
  w->sample_in_byte = 0;
  w->cur_delay = -1;
  w->ninv = 0;
  int delay_in_samples = (int)(delay_at_start * s->sample_rate); /* New_parameters::delay_in_samples is int */
  if (s->bps == 2) {
    int sr = s->sample_rate, f = s->tsys_freq;
    int tc = (int)floor(delay_in_samples + 0.5);
    tc %= (sr / f);
    while (tc < 0) tc += sr / f;
    w->tsys_on = (tc < (sr / (2 * f)));
    tc %= (sr / (2 * f));
    tc = ((sr / (2 * f)) - tc);
    tc /= 4;
    w->tsys_count = tc;
  }
}

/* bit2float(): returns the new sample_in_byte, advances *readp (327-424) */
static int b2f_unpack(b2f_t *w, const unsigned char *in, float *out, int start, int nsamples, uint64_t *readp) {
  uint64_t read = *readp;
  int iout = 0;
  if (w->bps == 2) {
    int stw = nsamples < 4 - start ? nsamples : 4 - start;
    unsigned char byte = in[read];
    for (int k = 0; k < stw; k++) out[iout + k] = SAMPLE_MS[(byte >> (2 * (start + k))) & 3];
    if (w->tsys_on)
      w->stats.on[byte]++;
    else
      w->stats.off[byte]++;
    if (--w->tsys_count == 0) {
      w->tsys_count = (w->sr / (2 * w->tsys_freq)) / 4;
      w->tsys_on = !w->tsys_on;
    }
    nsamples -= stw;
    iout += stw;
    if (stw + start == 4)
      read++;
    else
      return start + stw;
    int nbytes = nsamples / 4;
    for (int b = 0; b < nbytes; b++) {
      byte = in[read];
      for (int k = 0; k < 4; k++) out[iout + k] = SAMPLE_MS[(byte >> (2 * k)) & 3];
      if (w->tsys_on)
        w->stats.on[byte]++;
      else
        w->stats.off[byte]++;
      if (--w->tsys_count == 0) {
        w->tsys_count = (w->sr / (2 * w->tsys_freq)) / 4;
        w->tsys_on = !w->tsys_on;
      }
      iout += 4;
      read++;
    }
    nsamples -= nbytes * 4;
    if (nsamples > 0) {
      byte = in[read];
      for (int k = 0; k < nsamples; k++) out[iout + k] = SAMPLE_MS[(byte >> (2 * k)) & 3];
      *readp = read;
      return nsamples;
    }
  } else {
    int stw = nsamples < 8 - start ? nsamples : 8 - start;
    unsigned char byte = in[read];
    for (int k = 0; k < stw; k++) out[iout + k] = SAMPLE_M[(byte >> (start + k)) & 1];
    w->stats.on[byte]++;
    nsamples -= stw;
    iout += stw;
    if (stw + start == 8)
      read++;
    else
      return start + stw;
    int nbytes = nsamples / 8;
    for (int b = 0; b < nbytes; b++) {
      byte = in[read];
      for (int k = 0; k < 8; k++) out[iout + k] = SAMPLE_M[(byte >> k) & 1];
      w->stats.on[byte]++;
      iout += 8;
      read++;
    }
    nsamples -= nbytes * 8;
    if (nsamples > 0) {
      byte = in[read];
      for (int k = 0; k < nsamples; k++) out[iout + k] = SAMPLE_M[(byte >> k) & 1];
      *readp = read;
      return nsamples;
    }
  }
  *readp = read;
  return 0;
}

/* One integration: consumes protocol bytes from in[*pos, n) and fills
   out[n_ffts * fft_size] (do_task, 36-197; buffers of nfft_max blocks). */
static void b2f_integration(b2f_t *w, const unsigned char *in, size_t n, uint64_t *pos, float *out) {
  uint64_t read = *pos;
  const uint64_t write = n;
  int current_fft = 0;
  while (current_fft < w->n_ffts) {
    int nfft = w->nfft_max < w->n_ffts - current_fft ? w->nfft_max : w->n_ffts - current_fft;
    size_t size = (size_t)nfft * w->fft_size;
    float *ob = out + (size_t)current_fft * w->fft_size;
    size_t out_index = 0;
    while (out_index != size) {
      if (w->sample_in_byte >= 8) die("bit2float: sample_in_byte out of range");
      switch (w->state) {
        case B_IDLE: {
          if (write - read < 3) die("protocol ended before the integration was complete");
          unsigned char header = in[read++];
          if (header == HEADER_DATA) {
            w->bytes_left = in[read++];
            w->bytes_left |= (size_t)in[read++] << 8;
            w->state = B_SEND_DATA;
          } else if (header == HEADER_DELAY) {
            int8_t nd = (int8_t)in[read++];
            if (w->cur_delay < 0) {
              w->sample_in_byte = nd;
            } else {
              int diff = nd - w->cur_delay;
              if (diff == -1 || diff > 1) {
                ob[out_index++] = 0.0f; /* insert a sample */
              } else {
                if (w->sample_in_byte != 0) die("bit2float: drop with sample_in_byte != 0");
                w->sample_in_byte = 1; /* remove a sample */
              }
            }
            w->cur_delay = nd;
          } else if (header == HEADER_INVALID) {
            w->invalid_left = in[read++];
            w->invalid_left |= (size_t)in[read++] << 8;
            w->stats.ninvalid += (int)w->invalid_left;
            if (w->ninv == w->capinv) {
              w->capinv = w->capinv * 2 + 16;
              w->inv = xrealloc(w->inv, w->capinv * sizeof(inval_t));
            }
            w->inv[w->ninv].begin = current_fft * w->fft_size + (int)out_index;
            w->inv[w->ninv].n = (int)w->invalid_left;
            w->ninv++;
            w->state = B_SEND_INVALID;
          } else {
            die("bit2float: invalid header");
          }
          break;
        }
        case B_SEND_INVALID: {
          size_t freeb = size - out_index;
          size_t itw = freeb < w->invalid_left ? freeb : w->invalid_left;
          if (w->sample_in_byte > 0) {
            size_t drop = w->sample_in_byte < itw ? w->sample_in_byte : itw;
            w->sample_in_byte -= drop;
            itw -= drop;
            w->invalid_left -= drop;
          }
          if (itw > 0) {
            memset(ob + out_index, 0, itw * sizeof(float));
            w->invalid_left -= itw;
            out_index += itw;
          }
          if (w->invalid_left == 0) w->state = B_IDLE;
          break;
        }
        case B_SEND_DATA: {
          if (read == write) die("protocol ended inside a data block");
          int spb = 8 / w->bps;
          size_t freeb = size - out_index;
          size_t bin = (write - read) < w->bytes_left ? (write - read) : w->bytes_left;
          size_t a = bin * spb - w->sample_in_byte;
          size_t stw = a < freeb ? a : freeb;
          w->bytes_left -= (stw + w->sample_in_byte) / spb;
          w->sample_in_byte = b2f_unpack(w, in, ob + out_index, (int)w->sample_in_byte, (int)stw, &read);
          out_index += stw;
          if (w->bytes_left == 0) {
            if (w->sample_in_byte != 0) die("bit2float: data block ended mid-byte");
            w->state = B_IDLE;
          }
          break;
        }
        case B_PURGE: {
          size_t adv = (write - read) < w->bytes_left ? (write - read) : w->bytes_left;
          read += adv;
          w->bytes_left -= adv;
          if (w->bytes_left == 0 && write - read > 0) {
            switch (in[read]) {
              case HEADER_ENDSTREAM:
                read += 1;
                w->state = B_IDLE;
                break;
              case HEADER_DELAY:
                if (write - read >= 2) read += 2;
                break;
              case HEADER_INVALID:
                if (write - read >= 3) read += 3;
                break;
              case HEADER_DATA:
                if (write - read >= 3) {
                  read += 1;
                  w->bytes_left = in[read++];
                  w->bytes_left |= (size_t)in[read++] << 8;
                }
                break;
            }
          } else if (w->bytes_left == 0) {
            die("protocol ended while skipping the previous integration");
          }
          break;
        }
      }
    }
    current_fft += nfft;
  }
  w->state = B_PURGE;
  *pos = read;
}

/* --------------------------------------------------------- delay correction ---
 * Delay_correction (sfxc/src/delay_correction.cc:21-259, 300-353) */
typedef struct {
  int Nd, rot, cor, stride, oversamp, bw, sr, sb, window, flipsb;
  int64_t channel_freq;
  double LO_offset, start_phase;
  int output_offset, temp_fft_offset, n_blocks;
  double *win; /* float-rounded in precision 32 */
  fftplan_t *pNd2, *pNd, *pr2, *pr;
} dc_t;

static void dc_setup(dc_t *d, const job_t *j, const stream_t *s) {
  d->Nd = j->Nd;
  d->cor = 2 * j->M;
  d->rot = (int)(((uint64_t)d->cor * (uint64_t)s->sample_rate) / j->sample_rate);
  d->stride = d->cor / 2 + 4;
  d->sr = s->sample_rate;
  d->bw = s->bandwidth;
  d->oversamp = (int)round(s->sample_rate / (2 * (double)s->bandwidth));
  d->sb = s->sideband == 'L' ? -1 : 1;
  d->channel_freq = s->channel_freq;
  d->window = j->window;
  d->flipsb = j->sideband != s->sideband;
  d->LO_offset = s->LO_offset;
  int n = d->rot;
  d->win = xmalloc(n * sizeof(double));
  for (int i = 0; i < n; i++) { /* create_window (300-341) */
    double v = 0;
    switch (j->window) {
      case WINDOW_NONE: v = i < n / 2 ? 1 : 0; break;
      case WINDOW_RECT: v = (i >= n / 4 && i < 3 * n / 4) ? 1 : 0; break;
      case WINDOW_COS: v = sin(M_PI * i / (n - 1)); break;
      case WINDOW_HAMMING: v = 0.54 - 0.46 * cos(2 * M_PI * i / (n - 1)); break;
      case WINDOW_HANN: v = 0.5 * (1 - cos(2 * M_PI * i / (n - 1))); break;
      default: die("invalid window");
    }
    d->win[i] = st(v);
  }
  /* output offsets for mixed bandwidths (226-241) */
  int64_t delta, freq = s->channel_freq;
  if (j->sideband != s->sideband) freq += d->sb * (int64_t)s->bandwidth;
  if (j->sideband == 'L')
    delta = freq - j->channel_freq;
  else
    delta = j->channel_freq - freq;
  if (delta > 0) {
    d->output_offset = (int)(delta * d->cor / j->sample_rate);
    d->temp_fft_offset = 0;
  } else {
    d->output_offset = 0;
    d->temp_fft_offset = (int)(-delta * d->cor / j->sample_rate);
  }
  d->pNd2 = fft_plan(d->Nd / 2);
  d->pNd = fft_plan(d->Nd);
  d->pr2 = fft_plan(d->rot / 2);
  d->pr = fft_plan(d->rot);
}

/* Corrects one integration of float samples x[n_blocks*Nd] into rows of
   'stride' complex values (re, im interleaved doubles).  Returns the row count.
   Time stamps follow the reference: block b starts at start + b*Nd samples. */
static int dc_integration(dc_t *d, const job_t *j, const akima_t *a, ticks_t start, int n_blocks, const float *x,
                          double *rows) {
  const int Nd = d->Nd, half = Nd / 2;
  int tps = t_sample_rate(d->sr);
  ticks_t fft_length = t_from_usec((double)Nd / (d->sr / 1000000));
  ticks_t half_len = t_div(fft_length, 2);
  double dt = t_diff(start, j->experiment_start);
  double sp = d->LO_offset * (dt - trunc(dt)) + (d->LO_offset - trunc(d->LO_offset)) * trunc(dt);
  d->start_phase = sp - floor(sp);
  size_t nsamp = (size_t)n_blocks * Nd;
  double *ts = xmalloc(nsamp * sizeof(double)); /* fringe-stopped series (float-rounded in p32) */
  double *fr = xmalloc((Nd / 2 + 1) * 8), *fi = xmalloc((Nd / 2 + 1) * 8);
  double *zr = xmalloc(Nd * 8), *zi = xmalloc(Nd * 8);
  double *wre = xmalloc(d->rot * 8), *wim = xmalloc(d->rot * 8);
  double *blk = xmalloc(Nd * 8);
  const double dfr = (double)d->sr / Nd;
  const double mult = -d->sb * 2.0 * M_PI;
  const double center_freq = d->channel_freq + d->sb * d->bw * 0.5 + d->LO_offset;
  for (int b = 0; b < n_blocks; b++) {
    ticks_t ct = start + (ticks_t)b * Nd * tps;
    double delay = dt_delay(a, ct + half_len);
    double dis = delay * d->sr;
    int integer_delay = (int)floor(dis + .5);
    double frac = dis - integer_delay;
    /* fractional_bit_shift (82-137) */
    for (int i = 0; i < Nd; i++) blk[i] = x[(size_t)b * Nd + i];
    fft_r2c(d->pNd2, d->pNd, blk, fr, fi, wre, wim);
    for (int i = 0; i <= half; i++) {
      fr[i] = st(fr[i]);
      fi[i] = st(fi[i]);
    }
    fr[0] = st(fr[0] * 0.5);
    fi[0] = st(fi[0] * 0.5);
    fr[half] = st(fr[half] * 0.5);
    fi[half] = st(fi[half] * 0.5);
    const double tmp1 = -2.0 * M_PI * frac / d->sr;
    const double tmp2 = M_PI * (integer_delay & (4 * d->oversamp - 1)) / (2 * d->oversamp);
    const double constant_term = tmp2 - tmp1 * 0.5 * d->bw;
    const double linear_term = tmp1 * dfr;
    double temp = sin(linear_term / 2);
    double aa = 2 * temp * temp, bb = sin(linear_term);
    double cp, sp2;
    sincos(constant_term, &sp2, &cp);
    for (int i = 0; i <= half; i++) {
      double er = st(cp), ei = st(-sp2); /* complex<FLOAT>(cos, -sin) */
      double pr, pi;
      if (g_f64) {
        pr = er * fr[i] - ei * fi[i];
        pi = er * fi[i] + ei * fr[i];
      } else {
        float a1 = (float)er, b1 = (float)ei, c1 = (float)fr[i], d1 = (float)fi[i];
        pr = (float)((float)(a1 * c1) - (float)(b1 * d1));
        pi = (float)((float)(a1 * d1) + (float)(b1 * c1));
      }
      zr[i] = pr;
      zi[i] = pi;
      temp = sp2 - (aa * sp2 - bb * cp);
      cp = cp - (aa * cp + bb * sp2);
      sp2 = temp;
    }
    for (int i = half + 1; i < Nd; i++) zr[i] = zi[i] = 0.0;
    fft_c(d->pNd, zr, zi, +1);
    for (int i = 0; i < Nd; i++) {
      zr[i] = st(zr[i]);
      zi[i] = st(zi[i]);
    }
    /* fringe_stopping (139-184) */
    double lo_phase = d->start_phase + d->LO_offset * t_diff(ct, start);
    double phi = center_freq * dt_delay(a, ct) + lo_phase + dt_phase(a, ct) / (2 * M_PI);
    double floor_phi = floor(phi);
    phi = mult * (phi - floor_phi);
    double phi_end = center_freq * dt_delay(a, ct + fft_length) + lo_phase +
                     t_get_time(fft_length) * d->LO_offset + dt_phase(a, ct + fft_length) / (2 * M_PI);
    phi_end = mult * (phi_end - floor_phi);
    double delta_phi = (phi_end - phi) / Nd;
    double amplitude = dt_amplitude(a, ct + half_len);
    temp = sin(delta_phi / 2);
    aa = 2 * temp * temp;
    bb = sin(delta_phi);
    double sphi, cphi;
    sincos(phi, &sphi, &cphi);
    sphi *= amplitude;
    cphi *= amplitude;
    for (int i = 0; i < Nd; i++) {
      ts[(size_t)b * Nd + i] = st(zr[i] * cphi + zi[i] * sphi);
      temp = sphi - (aa * sphi - bb * cphi);
      cphi = cphi - (aa * cphi + bb * sphi);
      sphi = temp;
    }
  }
  /* windowed FFTs over the continuous series (57-75) */
  const int rot = d->rot, hop = rot / 2;
  const int nper = d->window == WINDOW_NONE ? hop : rot;
  int nrows = (int)(nsamp / hop) - (d->window != WINDOW_NONE ? 1 : 0);
  int tfsize = (d->cor > rot ? d->cor : rot) / 2 + 4;
  double *tf_re = xmalloc(tfsize * 8), *tf_im = xmalloc(tfsize * 8);
  double *ore = xmalloc((rot / 2 + 1) * 8), *oim = xmalloc((rot / 2 + 1) * 8);
  double *tb = xmalloc(rot * 8);
  for (int r = 0; r < nrows; r++) {
    size_t s0 = (size_t)r * hop;
    for (int i = 0; i < rot; i++) {
      double v = i < nper ? st(ts[s0 + i] * d->win[i]) : 0.0;
      if (d->flipsb && (i % 2)) v = -v;
      tb[i] = v;
    }
    fft_r2c(d->pr2, d->pr, tb, ore, oim, wre, wim);
    for (int i = 0; i <= rot / 2; i++) {
      tf_re[d->temp_fft_offset + i] = st(ore[i]);
      tf_im[d->temp_fft_offset + i] = st(oim[i]);
    }
    double *row = rows + (size_t)r * d->stride * 2;
    for (int i = 0; i < d->stride; i++) {
      row[2 * i] = tf_re[d->output_offset + i];
      row[2 * i + 1] = tf_im[d->output_offset + i];
    }
  }
  free(ts); free(fr); free(fi); free(zr); free(zi); free(wre); free(wim); free(blk);
  free(tf_re); free(tf_im); free(ore); free(oim); free(tb);
  return nrows;
}

/* ----------------------------------------------------------- correlation ---
 * Correlation_core (sfxc/src/correlation_core.cc:134-171 baselines, 241-273
 * X-step, 275-314 normalisation, 316-477 output, 480-513 tsys, 516-559
 * sub-integrations, 599-665 flagged samples), Correlation_core_pulsar
 * (sfxc/src/correlation_core_pulsar.cc:13-99 setup, 101-146, 210-238 bins). */
typedef struct {
  int a, b;
} bl_t;

static int make_baselines(const job_t *j, bl_t *bl) {
  int n = 0, N = j->nstreams;
  for (int i = 0; i < N; i++) bl[n++] = (bl_t){i, i};
  for (int i = 0; i < N; i++)
    for (int k = i + 1; k < N; k++) {
      int s1 = j->streams[i].station_number, s2 = j->streams[k].station_number;
      if (s1 == s2) continue;
      if (j->reference_station >= 0 && j->reference_station != s1 && j->reference_station != s2) continue;
      if (s1 < s2)
        bl[n++] = (bl_t){i, k};
      else
        bl[n++] = (bl_t){k, i};
    }
  return n;
}

static void find_invalid(const job_t *j, const bl_t *bl, int nbl, b2f_t *w, int64_t (*nfl)[2]) {
  for (int b = j->nstreams; b < nbl; b++) {
    int st_[2] = {bl[b].a, bl[b].b};
    double scale[2] = {j->streams[st_[0]].sample_rate * 1. / j->sample_rate,
                       j->streams[st_[1]].sample_rate * 1. / j->sample_rate};
    b2f_t *iw[2] = {&w[st_[0]], &w[st_[1]]};
    int index[2] = {0, 0}, nflagged[2] = {0, 0};
    int is[2] = {INT_MAX, INT_MAX}, ie[2] = {INT_MAX, INT_MAX};
    int isz[2] = {iw[0]->ninv, iw[1]->ninv};
    for (int i = 0; i < 2; i++)
      if (isz[i] > 0) {
        is[i] = (int)floor(iw[i]->inv[0].begin / scale[i]);
        ie[i] = is[i] + (int)floor(iw[i]->inv[index[i]].n / scale[i]);
        index[i]++;
      }
    int i = is[0] < is[1] ? 0 : 1;
    while (is[i] < INT_MAX) {
      if (is[0] == is[1]) {
        if (ie[0] == ie[1]) {
          is[0] = ie[0] + 1;
          is[1] = ie[1] + 1;
        } else {
          int k = ie[0] < ie[1] ? 0 : 1;
          is[1 - k] = ie[k];
          is[k] = ie[k] + 1;
        }
      } else if (ie[i] < is[1 - i]) {
        nflagged[1 - i] += ie[i] - is[i];
        is[i] = ie[i] + 1;
      } else {
        nflagged[1 - i] += is[1 - i] - is[i];
        is[i] = is[1 - i];
      }
      for (int k = 0; k < 2; k++) {
        if (is[k] > ie[k]) {
          if (index[k] < isz[k]) {
            is[k] = (int)floor(iw[k]->inv[index[k]].begin / scale[k]);
            ie[k] = is[k] + (int)floor(iw[k]->inv[index[k]].n / scale[k]);
            index[k]++;
          } else {
            is[k] = INT_MAX;
            ie[k] = INT_MAX;
          }
        }
      }
      i = is[0] < is[1] ? 0 : 1;
    }
    nfl[b][0] += nflagged[0];
    nfl[b][1] += nflagged[1];
  }
}

/* acc: nbl x (M+1) complex as double pairs.  Normalises in place. */
static void normalize(const job_t *j, const bl_t *bl, int nbl, double *acc, b2f_t *w, int64_t (*nfl)[2],
                      int nffts) {
  const int M = j->M, K = M + 1;
  double *norms = xmalloc(j->nstreams * 8);
  for (int i = 0; i < j->nstreams; i++) {
    double s = 0;
    for (int k = 0; k < K; k++) s += acc[((size_t)i * K + k) * 2];
    s /= M;
    if (s < 1) s = 1;
    norms[i] = s;
    for (int k = 0; k < K; k++) {
      acc[((size_t)i * K + k) * 2] = st(acc[((size_t)i * K + k) * 2] / s);
      acc[((size_t)i * K + k) * 2 + 1] = 0;
    }
  }
  const int64_t total = (int64_t)nffts * M;
  for (int b = j->nstreams; b < nbl; b++) {
    int l1[5], l2[5];
    stats_levels(&w[bl[b].a].stats, l1);
    stats_levels(&w[bl[b].b].stats, l2);
    int64_t v1 = total - l1[4], v2 = total - l2[4];
    double N1 = v1 > 0 ? 1 - nfl[b][0] * 1. / v1 : 1;
    double N2 = v2 > 0 ? 1 - nfl[b][1] * 1. / v2 : 1;
    double N = N1 * N2;
    if (N < 0.01) N = 1;
    double norm = st(sqrt(N * norms[bl[b].a] * norms[bl[b].b]));
    for (int k = 0; k < K; k++) {
      acc[((size_t)b * K + k) * 2] = st(acc[((size_t)b * K + k) * 2] / norm);
      acc[((size_t)b * K + k) * 2 + 1] = st(acc[((size_t)b * K + k) * 2 + 1] / norm);
    }
  }
  free(norms);
}

/* ---------------------------------------------------- spectral reduction ---
 * Correlation_core::integration_write for number_channels < fft size
 * (sfxc/src/correlation_core.cc:413-439) with create_window (760-810) and
 * create_mask (812-824): per baseline, optional normalisation to unit
 * amplitude, the mask, an unnormalised c2r FFT of 2M points (imaginary parts
 * of DC and Nyquist ignored), the lags folded to 2 nch, the lag window, an
 * r2c FFT of 2 nch points, and a division by 2M; every step stored in FP32 as
 * the reference's buffers are. */
static double lagwin_f(int type, int n, int i) { /* cos / hamming / hann (667-690) */
  switch (type) {
    case WINDOW_COS: return sin(M_PI * i / n);
    case WINDOW_HAMMING: return 0.54 - 0.46 * cos(2 * M_PI * i / n);
    default: return 0.5 * (1 - cos(2 * M_PI * i / n));
  }
}
static double lagwin_conv(int type, int n, int i) { /* convolve (692-706) */
  double sum = 0.0;
  i += n / 2;
  for (int q = 0; q <= n; q++) {
    if (i - q < 0 || i - q > n) continue;
    sum += lagwin_f(type, n, q) * lagwin_f(type, n, i - q);
  }
  return sum;
}
static double *lag_window_of(const job_t *j) {
  static double *cache = NULL;
  static int cn = -1, cm = -1, ct = -1;
  const int n = 2 * j->number_channels, m = 2 * j->M;
  if (j->lag_window) return j->lag_window;
  if (cache && cn == n && cm == m && ct == j->window) return cache;
  free(cache);
  cache = xmalloc(n * sizeof(double));
  cn = n, cm = m, ct = j->window;
  if (j->window == WINDOW_NONE || j->window == WINDOW_RECT) {
    cache[0] = 1.;
    for (int i = 1; i < n / 2; i++) cache[i] = cache[n - i] = st((1. - 2. * i / n) / (1. - 2. * i / m));
    cache[n / 2] = 0.;
  } else {
    const int r = m / n; /* integer ratio, as in the reference */
    cache[0] = st(r * lagwin_conv(j->window, n, n / 2) / lagwin_conv(j->window, m, m / 2));
    for (int i = 1; i < n / 2; i++)
      cache[i] = cache[n - i] = st(r * lagwin_conv(j->window, n, n / 2 + i) / lagwin_conv(j->window, m, m / 2 + i));
    cache[n / 2] = st(r * lagwin_conv(j->window, n, n) / lagwin_conv(j->window, m, (n + m) / 2));
  }
  return cache;
}
/* x: M + 1 complex (normalised visibilities), y: nch + 1 complex */
static void reduce_spectrum(const job_t *j, const double *x, double *y) {
  const int M = j->M, n2 = 2 * M, nch = j->number_channels, m2 = 2 * nch;
  static fftplan_t *p2m = NULL, *p2n = NULL;
  if (!p2m || p2m->n != n2) p2m = fft_plan(n2); /* plans are kept (one job per process) */
  if (!p2n || p2n->n != m2) p2n = fft_plan(m2);
  double *re = xmalloc(n2 * 8), *im = xmalloc(n2 * 8);
  for (int k = 0; k <= M; k++) {
    double a = x[2 * k], b = x[2 * k + 1];
    if (j->mask_normalize) {
      const double mag = st(sqrt(a * a + b * b));
      if (mag != 0.0) a = st(a / mag), b = st(b / mag);
    }
    const double mv = j->mask ? j->mask[k] : 1.0;
    re[k] = st(a * mv);
    im[k] = st(b * mv);
  }
  im[0] = 0, im[M] = 0;
  for (int k = M + 1; k < n2; k++) re[k] = re[n2 - k], im[k] = -im[n2 - k];
  fft_c(p2m, re, im, +1);
  for (int i = 0; i < n2; i++) re[i] = st(re[i]);
  double *lag = xmalloc(m2 * 8), *li = xmalloc(m2 * 8);
  const double *w = lag_window_of(j);
  for (int q = 0; q < m2; q++) {
    double v = q < nch ? re[q] : q == nch ? st(st(re[nch] + re[n2 - nch]) / 2) : re[n2 - nch + (q - nch)];
    lag[q] = st(v * w[q]);
    li[q] = 0;
  }
  fft_c(p2n, lag, li, -1);
  for (int q = 0; q <= nch; q++) {
    y[2 * q] = st(st(lag[q]) / (double)(float)n2);
    y[2 * q + 1] = st(st(li[q]) / (double)(float)n2);
  }
  free(re), free(im), free(lag), free(li);
}

/* -------------------------------------------------- extra phase centres ---
 * Correlation_core::create_weights (sfxc/src/correlation_core.cc:708-744):
 * the autocorrelation of the zero-padded window over 2M - 1 points, through
 * an FP32 r2c / c2r pair of 4M points, normalised at lag 0. */
static double pc_window_f(int type, int n, int i) { /* rect / cos / hamming / hann (667-690) */
  switch (type) {
    case WINDOW_NONE:
    case WINDOW_RECT: return (i >= n / 4 && i < (3 * n) / 4) ? 1.0 : 0.0;
    case WINDOW_COS: return sin(M_PI * i / n);
    case WINDOW_HAMMING: return 0.54 - 0.46 * cos(2 * M_PI * i / n);
    default: return 0.5 * (1 - cos(2 * M_PI * i / n));
  }
}
static const double *pc_weights(const job_t *j) {
  static double *w = NULL;
  if (w) return w;
  const int n = j->M, n4 = 4 * n;
  fftplan_t *p = fft_plan(n4);
  double *re = xmalloc(n4 * 8), *im = xmalloc(n4 * 8);
  for (int i = 0; i < 2 * n; i++) re[i] = st(pc_window_f(j->window, 2 * n - 1, i));
  fft_c(p, re, im, -1);
  for (int q = 0; q <= 2 * n; q++) { /* conj(F) F in FP32 */
    const double a = st(re[q]), b = st(im[q]);
    re[q] = st(st(a * a) + st(b * b));
    im[q] = 0;
  }
  for (int q = 2 * n + 1; q < n4; q++) re[q] = re[n4 - q], im[q] = 0;
  im[0] = im[2 * n] = 0;
  fft_c(p, re, im, +1);
  w = xmalloc(n * 8);
  const double t0 = st(re[0]);
  for (int i = 0; i < n; i++) w[i] = st(st(re[i]) / t0);
  free(re), free(im);
  return w;
}
/* Correlation_core::uvshift (sfxc/src/correlation_core.cc:561-593): one
   baseline's sub-integration spectrum in[K] rotated by the residual delay of
   an extra phase centre and added to out[K]; FP32 products, FP64 phase
   recurrence, as the reference. */
static void uvshift_add(const job_t *j, const double *in, double *out, double dd1, double dd2, double r1,
                        double r2) {
  const int K = j->M + 1;
  const int sb = j->sideband == 'L' ? -1 : 1;
  const double base_freq = (double)j->channel_freq;
  const double dfreq = j->sample_rate / (2. * j->M);
  const double *weights = pc_weights(j);
  double amplitude = 1;
  const int lag = abs((int)round((dd1 - dd2) * j->sample_rate));
  if (lag < j->M && weights[lag] > 1e-4) amplitude = st(1. / weights[lag]);
  double phi = base_freq * (dd1 * (1 - r1) - dd2 * (1 - r2));
  phi = 2 * M_PI * sb * (phi - floor(phi));
  const double delta = 2 * M_PI * dfreq * (dd1 * (1 - r1) - dd2 * (1 - r2));
  double temp = sin(delta / 2);
  const double a = 2 * temp * temp, b = sin(delta);
  double c = cos(phi), s = sin(phi);
  for (int i = 0; i < K; i++) {
    const double xr = st(amplitude * in[2 * i]), xi = st(amplitude * in[2 * i + 1]);
    const double cf = st(c), sf = st(s);
    out[2 * i] = st(out[2 * i] + st(st(xr * cf) - st(xi * sf)));
    out[2 * i + 1] = st(out[2 * i + 1] + st(st(xr * sf) + st(xi * cf)));
    temp = s - (a * s - b * c);
    c = c - (a * c + b * s);
    s = temp;
  }
}

static void write_integration(const job_t *j, const bl_t *bl, int nbl, const double *acc, b2f_t *w,
                              int64_t (*nfl)[2], int nffts, int integration, int32_t sourcenr, int centre,
                              bytes_t *out, bytes_t *out64) {
  const int M = j->M, K = M + 1, N = j->nstreams;
  bpush(out, &sourcenr, 4);
  /* stations in stream order, with the first stream of each
   * (Correlation_core::integration_write, sfxc/src/correlation_core.cc:350-364) */
  int stations[512], first[512], nst = 0;
  for (int i = 0; i < N; i++) {
    int s = j->streams[i].station_number, seen = 0;
    for (int k = 0; k < nst; k++) seen |= stations[k] == s;
    if (!seen) first[nst] = i, stations[nst++] = s;
  }
  const int npc = j->n_pc > 1 ? j->n_pc : 1;
  int32_t ts[4] = {j->integration_nr + integration, nbl, nst, N};
  bpush(out, ts, 16);
  for (int k = 0; k < nst; k++) {
    int32_t h[2] = {stations[k], 0};
    double uvw[3] = {0, 0, 0};
    if (j->uvw) {
      const size_t o = (((size_t)integration * N + first[k]) * npc + centre) * 3;
      if (o + 3 > j->n_uvw) die("uvw file too short");
      memcpy(uvw, j->uvw + o, sizeof(uvw));
    }
    bpush(out, h, 8);
    bpush(out, uvw, 24);
  }
  for (int i = 0; i < N; i++) {
    unsigned char h[4] = {(unsigned char)j->streams[i].station_number, (unsigned char)j->frequency_nr,
                          (unsigned char)(j->sideband == 'L' ? 0 : 1),
                          (unsigned char)(j->streams[i].pol == 'R' ? 0 : 1)};
    int lv[5];
    stats_levels(&w[i].stats, lv);
    int32_t l[5];
    if (w[i].bps == 2) {
      l[0] = lv[0]; l[1] = lv[1]; l[2] = lv[2]; l[3] = lv[3];
    } else {
      l[0] = 0; l[1] = lv[0]; l[2] = lv[1]; l[3] = 0;
    }
    l[4] = lv[4];
    bpush(out, h, 4);
    bpush(out, l, 20);
  }
  const int64_t total = (int64_t)nffts * M;
  for (int b = 0; b < nbl; b++) {
    int lv[5];
    stats_levels(&w[bl[b].a].stats, lv);
    int64_t wgt = bl[b].a == bl[b].b ? total - lv[4] : total - lv[4] - nfl[b][0];
    if (wgt < 0) wgt = 0;
    int32_t w32 = (int32_t)wgt;
    unsigned char h[4];
    h[0] = (unsigned char)j->streams[bl[b].a].station_number;
    h[1] = (unsigned char)j->streams[bl[b].b].station_number;
    h[2] = (unsigned char)((j->streams[bl[b].a].pol == 'R' ? 0 : 1) | ((j->streams[bl[b].b].pol == 'R' ? 0 : 1) << 1) |
                           ((j->sideband == 'U' ? 1 : 0) << 2) | ((j->frequency_nr & 31) << 3));
    h[3] = ' ';
    bpush(out, &w32, 4);
    bpush(out, h, 4);
    const double *x = acc + (size_t)b * K * 2;
    double *y = NULL;
    int Ko = K;
    if (j->number_channels != M) {
      Ko = j->number_channels + 1;
      y = xmalloc((size_t)Ko * 16);
      reduce_spectrum(j, x, y);
      x = y;
    }
    for (int k = 0; k < Ko; k++) {
      float v[2] = {(float)x[2 * k], (float)x[2 * k + 1]};
      bpush(out, v, 8);
      if (out64) bpush(out64, &x[2 * k], 16);
    }
    free(y);
  }
}

static void tsys_write(const job_t *j, ticks_t start, b2f_t *w, bytes_t *out) {
  for (int i = 0; i < j->nstreams; i++) {
    unsigned char h[4] = {(unsigned char)j->streams[i].station_number, (unsigned char)j->frequency_nr,
                          (unsigned char)(j->sideband == 'L' ? 0 : 1),
                          (unsigned char)(j->streams[i].pol == 'R' ? 0 : 1)};
    int ts[4];
    stats_tsys(&w[i].stats, ts);
    int64_t v[5] = {start, ts[0], ts[1], ts[2], ts[3]};
    bpush(out, h, 4);
    bpush(out, v, 40);
  }
}

/* X-step over rows of all streams. Products accumulate in float (p32) with the
   reference's sub-integration dumps at Delay_correction buffer boundaries, or
   in double (p64). */
static void xstep_rows(const job_t *j, const bl_t *bl, int nbl, double **rows, int stride, int r0, int r1,
                       double *acc) {
  const int K = j->M + 1;
  for (int r = r0; r < r1; r++) {
    for (int b = 0; b < nbl; b++) {
      const double *x = rows[bl[b].a] + (size_t)r * stride * 2;
      const double *y = rows[bl[b].b] + (size_t)r * stride * 2;
      double *ac = acc + (size_t)b * K * 2;
      for (int k = 0; k < K; k++) {
        double xr = x[2 * k], xi = x[2 * k + 1], yr = y[2 * k], yi = -y[2 * k + 1];
        if (g_f64) {
          ac[2 * k] += xr * yr - xi * yi;
          ac[2 * k + 1] += xr * yi + xi * yr;
        } else {
          float pr = (float)((float)((float)xr * (float)yr) - (float)((float)xi * (float)yi));
          float pi = (float)((float)((float)xr * (float)yi) + (float)((float)xi * (float)yr));
          ac[2 * k] = (float)((float)ac[2 * k] + pr);
          ac[2 * k + 1] = (float)((float)ac[2 * k + 1] + pi);
        }
      }
    }
  }
}

/* ------------------------------------------------------------ job parsing */
typedef struct {
  char *key;
  int nv;
  char **v;
} kv_t;
typedef struct {
  kv_t *e;
  int n;
} kvs_t;
static kvs_t read_job(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) die("cannot open job");
  kvs_t r = {0, 0};
  char line[1 << 16];
  while (fgets(line, sizeof(line), f)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    r.e = xrealloc(r.e, (r.n + 1) * sizeof(kv_t));
    kv_t *e = &r.e[r.n++];
    e->nv = 0;
    e->v = NULL;
    char *save = NULL;
    char *tok = strtok_r(line, " \t\r\n", &save);
    e->key = strdup(tok ? tok : "");
    while ((tok = strtok_r(NULL, " \t\r\n", &save))) {
      e->v = xrealloc(e->v, (e->nv + 1) * sizeof(char *));
      e->v[e->nv++] = strdup(tok);
    }
  }
  fclose(f);
  return r;
}
static kv_t *kv_get(const kvs_t *k, const char *key, int idx) {
  int c = 0;
  for (int i = 0; i < k->n; i++)
    if (!strcmp(k->e[i].key, key)) {
      if (c == idx) return &k->e[i];
      c++;
    }
  return NULL;
}
static kv_t *kv_must(const kvs_t *k, const char *key, int idx) {
  kv_t *e = kv_get(k, key, idx);
  if (!e) {
    fprintf(stderr, "missing key %s\n", key);
    die("bad job");
  }
  return e;
}
static int kv_count(const kvs_t *k, const char *key) {
  int c = 0;
  for (int i = 0; i < k->n; i++) c += !strcmp(k->e[i].key, key);
  return c;
}
static long long kv_ll(const kvs_t *k, const char *key) { return atoll(kv_must(k, key, 0)->v[0]); }
static double kv_d(const kvs_t *k, const char *key) { return strtod(kv_must(k, key, 0)->v[0], NULL); }

static unsigned char *read_all(const char *path, size_t *n) {
  FILE *f = fopen(path, "rb");
  if (!f) die("cannot open input file");
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char *p = xmalloc(sz + 1);
  if (sz && fread(p, 1, sz, f) != (size_t)sz) die("short read");
  fclose(f);
  *n = sz;
  return p;
}
static void write_all(const char *path, const void *p, size_t n) {
  FILE *f = fopen(path, "wb");
  if (!f) die("cannot write output");
  if (n) fwrite(p, 1, n, f);
  fclose(f);
}

static void load_table(const kvs_t *k, int st_, deltable_t *t) {
  deltable_read(t, kv_must(k, "delfile", st_)->v[0]);
  kv_t *c = kv_get(k, "clock", st_);
  t->clock_offset = 0;
  t->clock_rate = 0;
  t->clock_epoch = 0;
  if (c) {
    t->clock_offset = strtod(c->v[0], NULL);
    t->clock_rate = strtod(c->v[1], NULL);
    t->clock_epoch = atoll(c->v[2]);
  }
}

static int mode_delays(const kvs_t *k, const char *outp) {
  deltable_t t;
  load_table(k, 0, &t);
  ticks_t s0 = kv_ll(k, "start_ticks"), s1 = kv_ll(k, "stop_ticks");
  int sr = (int)kv_ll(k, "sample_rate"), bps = (int)kv_ll(k, "bits_per_sample");
  akima_t a;
  akima_create(&a, &t, s0, s1 - s0);
  dlist_t l = {0};
  interval_delays(&a, s0, s1, sr, bps, &l);
  FILE *f = fopen(outp, "w");
  for (int i = 0; i < l.n; i++) fprintf(f, "%lld %d %d\n", (long long)l.v[i].time, l.v[i].bytes, l.v[i].rem);
  int np = kv_count(k, "probe");
  for (int i = 0; i < np; i++) {
    ticks_t pt = atoll(kv_must(k, "probe", i)->v[0]);
    fprintf(f, "P %lld %.17g %.17g %.17g %.17g\n", (long long)pt, dt_delay(&a, pt), dt_rate(&a, pt),
            dt_phase(&a, pt), dt_amplitude(&a, pt));
  }
  fclose(f);
  return 0;
}

static int mode_protocol(const kvs_t *k, const char *outp) {
  int sr = (int)kv_ll(k, "sample_rate"), bps = (int)kv_ll(k, "bits_per_sample");
  double integr = kv_d(k, "integr_time_us");
  size_t n;
  unsigned char *blob = read_all(kv_must(k, "blockfile", 0)->v[0], &n);
  int nb = kv_count(k, "block");
  cblock_t *blocks = xmalloc(nb * sizeof(cblock_t));
  for (int b = 0; b < nb; b++) {
    kv_t *e = kv_must(k, "block", b);
    blocks[b].start = atoll(e->v[0]);
    blocks[b].data = blob + atoll(e->v[1]);
    blocks[b].size = atoi(e->v[2]);
    blocks[b].ninv = (e->nv - 3) / 2;
    blocks[b].inv = xmalloc((blocks[b].ninv + 1) * sizeof(inval_t));
    for (int q = 0; q < blocks[b].ninv; q++) {
      blocks[b].inv[q].begin = atoi(e->v[3 + 2 * q]);
      blocks[b].inv[q].n = atoi(e->v[4 + 2 * q]);
    }
  }
  int ns = kv_count(k, "slice");
  pslice_t *sl = xmalloc(ns * sizeof(pslice_t));
  for (int s = 0; s < ns; s++) {
    kv_t *e = kv_must(k, "slice", s);
    sl[s].start = atoll(e->v[0]);
    sl[s].stop = atoll(e->v[1]);
    sl[s].nr_samples = atoll(e->v[2]);
    memset(&sl[s].delays, 0, sizeof(dlist_t));
    FILE *f = fopen(kv_must(k, "dlist", s)->v[0], "r");
    if (!f) die("cannot open delay list");
    char line[256];
    while (fgets(line, sizeof(line), f)) {
      if (line[0] == 'P' || line[0] == '\n') continue;
      long long t;
      int by, re;
      if (sscanf(line, "%lld %d %d", &t, &by, &re) == 3) dl_push(&sl[s].delays, (delay_t){t, by, re});
    }
    fclose(f);
  }
  bytes_t *outs = xmalloc(ns * sizeof(bytes_t));
  pcal_t pc;
  memset(&pc, 0, sizeof(pc));
  kv_t *pt = kv_get(k, "phasecal_ticks", 0);
  pc.T = pt ? atoll(pt->v[0]) : 0;
  pc.sr = sr, pc.bps = bps;
  pc.station = (unsigned char)kv_ll(k, "station_number");
  pc.sb = 1; /* the job's channel: USB, RCP, frequency 0 */
  protocol_write(blocks, nb, sl, ns, sr, bps, integr, outs, &pc);
  kv_t *po = kv_get(k, "phasecal_out", 0);
  if (po) write_all(po->v[0], pc.out.p, pc.out.n);
  FILE *f = fopen(outp, "wb");
  for (int s = 0; s < ns; s++) {
    uint64_t m = outs[s].n;
    fwrite(&m, 8, 1, f);
    if (m) fwrite(outs[s].p, 1, m, f);
  }
  fclose(f);
  return 0;
}

/* Channel_extractor_5 LUT semantics (sfxc/src/channel_extractor_5.cc:27-99) */
static int mode_extract(const kvs_t *k, const char *outp) {
  int N = (int)kv_ll(k, "word_bytes"), bps = (int)kv_ll(k, "bits_per_sample");
  int nsamples = (int)kv_ll(k, "nsamples");
  size_t n;
  unsigned char *in = read_all(kv_must(k, "infile", 0)->v[0], &n);
  int nsub = kv_count(k, "subband");
  FILE *f = fopen(outp, "wb");
  for (int s = 0; s < nsub; s++) {
    kv_t *e = kv_must(k, "subband", s);
    int fan_out = e->nv, spb = 8 / fan_out;
    /* lookup_table[n][byte] for this subband */
    unsigned char lut[64][256];
    memset(lut, 0, sizeof(lut));
    int low_bit = 1 << (8 - fan_out);
    for (int tr = 0; tr < fan_out; tr++) {
      int track = atoi(e->v[tr]);
      int nb = track / 8, bit = track % 8;
      for (int smp = 0; smp < 256; smp++)
        if ((smp >> bit) & 1) lut[nb][smp] |= (unsigned char)(low_bit << ((tr + 1) % bps));
      if ((tr + 1) % bps == 0) low_bit <<= bps;
    }
    int nout = nsamples * fan_out / 8;
    unsigned char *o = xmalloc(nout + 1);
    const unsigned char *ip = in;
    int op = 0;
    for (int smp = 0; smp < nsamples; smp += spb) {
      for (int i = 1; i < spb; i++) {
        for (int q = 0; q < N; q++) o[op] |= lut[q][*ip++];
        o[op] >>= fan_out;
      }
      for (int q = 0; q < N; q++) o[op] |= lut[q][*ip++];
      op++;
    }
    fwrite(o, 1, nout, f);
    free(o);
  }
  fclose(f);
  return 0;
}

static int mode_correlate(const kvs_t *k, const char *outdir) {
  job_t j;
  memset(&j, 0, sizeof(j));
  kv_t *pe = kv_get(k, "precision", 0);
  g_f64 = pe && atoi(pe->v[0]) == 64;
  j.experiment_start = kv_ll(k, "experiment_start_ticks");
  j.start = kv_ll(k, "start_ticks");
  j.integration_time_us = kv_d(k, "integration_time_us");
  j.sub_integration_time_us = kv_d(k, "sub_integration_time_us");
  j.number_channels = (int)kv_ll(k, "number_channels");
  j.Nd = (int)kv_ll(k, "fft_size_delaycor");
  j.M = (int)kv_ll(k, "fft_size_correlation");
  j.sample_rate = (int)kv_ll(k, "sample_rate");
  j.channel_freq = kv_ll(k, "channel_freq");
  j.bandwidth = (int)kv_ll(k, "bandwidth");
  j.sideband = kv_must(k, "sideband", 0)->v[0][0];
  j.frequency_nr = (int)kv_ll(k, "frequency_nr");
  j.pol = kv_must(k, "polarisation", 0)->v[0][0];
  j.cross_polarize = (int)kv_ll(k, "cross_polarize");
  j.reference_station = (int)kv_ll(k, "reference_station");
  j.window = (int)kv_ll(k, "window");
  j.integration_nr = (int)kv_ll(k, "integration_nr");
  j.n_integrations = (int)kv_ll(k, "n_integrations");
  kv_t *de = kv_get(k, "dump", 0);
  j.dump = de && atoi(de->v[0]);
  kv_t *db = kv_get(k, "dump_bins", 0);
  j.dump_bins = db && atoi(db->v[0]);
  if (j.number_channels < 2 || j.number_channels > j.M || (j.number_channels & (j.number_channels - 1)))
    die("number_channels must be a power of two no larger than the FFT size");
  kv_t *ph = kv_get(k, "phased_array", 0);
  j.phased = ph && atoi(ph->v[0]);
  kv_t *npc = kv_get(k, "n_phase_centers", 0);
  j.n_pc = npc ? atoi(npc->v[0]) : 1;
  if (j.n_pc < 1) die("n_phase_centers must be at least 1");
  j.pc_file = xmalloc(j.n_pc * sizeof(int));
  kv_t *pcf = kv_get(k, "pc_file_index", 0);
  if (pcf) {
    if (pcf->nv != j.n_pc) die("pc_file_index needs n_phase_centers values");
    for (int q = 0; q < j.n_pc; q++) j.pc_file[q] = atoi(pcf->v[q]);
  }
  kv_t *mn = kv_get(k, "mask_normalize", 0);
  j.mask_normalize = mn && atoi(mn->v[0]);
  /* mask and lag window: files of float32 values */
  kv_t *mk = kv_get(k, "mask", 0);
  if (mk) {
    size_t nb = 0;
    uint8_t *b = read_all(mk->v[0], &nb);
    if (nb != (size_t)(j.M + 1) * 4) die("mask needs fft_size_correlation + 1 float32 values");
    j.mask = xmalloc((j.M + 1) * sizeof(double));
    for (int q = 0; q <= j.M; q++) j.mask[q] = ((const float *)b)[q];
    free(b);
  }
  kv_t *uv = kv_get(k, "uvw", 0);
  if (uv) {
    size_t nb = 0;
    j.uvw = (double *)read_all(uv->v[0], &nb);
    j.n_uvw = nb / sizeof(double);
  }
  kv_t *lw = kv_get(k, "lag_window", 0);
  if (lw) {
    size_t nb = 0;
    uint8_t *b = read_all(lw->v[0], &nb);
    if (nb != (size_t)(2 * j.number_channels) * 4) die("lag_window needs 2 number_channels float32 values");
    j.lag_window = xmalloc(2 * j.number_channels * sizeof(double));
    for (int q = 0; q < 2 * j.number_channels; q++) j.lag_window[q] = ((const float *)b)[q];
    free(b);
  }
  j.nstreams = kv_count(k, "stream");
  j.streams = xmalloc(j.nstreams * sizeof(stream_t));
  for (int i = 0; i < j.nstreams; i++) {
    kv_t *e = kv_must(k, "stream", i);
    stream_t *s = &j.streams[i];
    s->station_number = atoi(e->v[0]);
    s->station_stream = atoi(e->v[1]);
    s->sample_rate = atoi(e->v[2]);
    s->channel_freq = atoll(e->v[3]);
    s->bandwidth = atoi(e->v[4]);
    s->sideband = e->v[5][0];
    s->pol = e->v[6][0];
    s->bps = atoi(e->v[7]);
    s->LO_offset = strtod(e->v[8], NULL);
    s->tsys_freq = atoi(e->v[9]);
    s->table = atoi(e->v[10]);
  }
  kv_t *ps = kv_get(k, "pulsar", 0);
  j.pulsar = ps != NULL;
  if (j.pulsar) {
    j.nbins = atoi(ps->v[0]) + 1;
    j.gate0 = strtod(ps->v[1], NULL);
    j.gate1 = strtod(ps->v[2], NULL);
    j.npolyco = kv_count(k, "polyco");
    j.polyco = xmalloc(j.npolyco * 40 * sizeof(double));
    for (int p = 0; p < j.npolyco; p++) {
      kv_t *e = kv_must(k, "polyco", p);
      double *pc = j.polyco + p * 40;
      for (int q = 0; q < 5; q++) pc[q] = strtod(e->v[q], NULL);
      pc[5] = e->nv - 5;
      for (int q = 5; q < e->nv && q < 39; q++) pc[q + 1] = strtod(e->v[q], NULL);
    }
  }
  int nst = kv_count(k, "delfile");
  deltable_t *tables = xmalloc(nst * sizeof(deltable_t));
  for (int s = 0; s < nst; s++) load_table(k, s, &tables[s]);
  /* protocol inputs */
  unsigned char **proto = xmalloc(j.nstreams * sizeof(void *));
  size_t *proto_n = xmalloc(j.nstreams * sizeof(size_t));
  size_t *proto_pos = xmalloc(j.nstreams * sizeof(size_t));
  for (int i = 0; i < j.nstreams; i++) {
    proto[i] = read_all(kv_must(k, "protocol", i)->v[0], &proto_n[i]);
    proto_pos[i] = 0;
  }
  bl_t *bl = xmalloc((size_t)j.nstreams * j.nstreams * sizeof(bl_t) + sizeof(bl_t));
  int nbl = make_baselines(&j, bl);
  const int M = j.M, K = M + 1, stride = M + 4;
  b2f_t *w = xmalloc(j.nstreams * sizeof(b2f_t));
  for (int i = 0; i < j.nstreams; i++) w[i].state = B_IDLE;
  bytes_t cor = {0}, cor64 = {0}, tsys = {0};
  char path[4096];
  snprintf(path, sizeof(path), "%s/stats.txt", outdir);
  FILE *statsf = fopen(path, "w");
  ticks_t tint = t_from_usec(j.integration_time_us);
  ticks_t tf = t_from_usec(M / (j.sample_rate / 1000000.));
  int nr_ffts = (int)floor((double)tint / tf);
  int nffts = nr_ffts - (j.window != WINDOW_NONE ? 1 : 0);
  int nsub = (int)floor((double)t_from_usec(j.sub_integration_time_us) / tf);
  for (int it = 0; it < j.n_integrations; it++) {
    ticks_t start = j.start + (ticks_t)it * tint;
    akima_t *ak = xmalloc(j.nstreams * sizeof(akima_t));
    double **rows = xmalloc(j.nstreams * sizeof(double *));
    int *chunk = NULL;
    int nchunks = 0;
    /* splines of the extra phase centres (index 1..n_pc-1), per stream */
    akima_t *akp = xmalloc((size_t)j.nstreams * j.n_pc * sizeof(akima_t));
    for (int i = 0; i < j.nstreams; i++)
      for (int c = 1; c < j.n_pc; c++) akima_create_pc(&akp[i * j.n_pc + c], &tables[j.streams[i].table], start, tint, c);
    for (int i = 0; i < j.nstreams; i++) {
      stream_t *s = &j.streams[i];
      akima_create(&ak[i], &tables[s->table], start, tint);
      b2f_set_parameters(&w[i], &j, s, dt_delay(&ak[i], start));
      float *x = xmalloc((size_t)w[i].n_ffts * j.Nd * sizeof(float));
      /* this integration's protocol is length-prefixed in the input file */
      uint64_t len;
      memcpy(&len, proto[i] + proto_pos[i], 8);
      /* the reference ring holds previous leftovers + this integration */
      static unsigned char *ring[4096];
      static size_t ring_n[4096], ring_r[4096];
      if (i >= 4096) die("too many streams");
      {
        size_t keep = ring_n[i] - ring_r[i];
        unsigned char *nr = xmalloc(keep + len + 1);
        if (keep) memcpy(nr, ring[i] + ring_r[i], keep);
        memcpy(nr + keep, proto[i] + proto_pos[i] + 8, len);
        free(ring[i]);
        ring[i] = nr;
        ring_n[i] = keep + len;
        ring_r[i] = 0;
      }
      proto_pos[i] += 8 + len;
      uint64_t rp = 0;
      b2f_integration(&w[i], ring[i], ring_n[i], &rp, x);
      ring_r[i] = rp;
      dc_t d;
      dc_setup(&d, &j, s);
      rows[i] = xmalloc((size_t)(nffts + 2) * stride * 2 * sizeof(double));
      int nr = dc_integration(&d, &j, &ak[i], start, w[i].n_ffts, x, rows[i]);
      if (nr != nffts) die("row count disagrees with the correlator's FFT count");
      if (i == 0) {
        /* Delay_correction output buffer sizes: one per bit2float buffer */
        int tb = 0, hop = d.rot / 2, done = 0;
        for (int c0 = 0; c0 < w[i].n_ffts; c0 += w[i].nfft_max) {
          int nb = w[i].nfft_max < w[i].n_ffts - c0 ? w[i].nfft_max : w[i].n_ffts - c0;
          int nc = (nb * j.Nd + tb) / hop - (j.window != WINDOW_NONE ? 1 : 0);
          tb += nb * j.Nd - nc * hop;
          if (nc > 0) {
            chunk = xrealloc(chunk, (nchunks + 1) * sizeof(int));
            chunk[nchunks++] = nc;
            done += nc;
          }
        }
      }
      if (j.dump) {
        snprintf(path, sizeof(path), "%s/unpacked_i%d_s%d.f32", outdir, it, i);
        write_all(path, x, (size_t)w[i].n_ffts * j.Nd * sizeof(float));
        float *rf = xmalloc((size_t)nffts * stride * 2 * sizeof(float));
        for (size_t q = 0; q < (size_t)nffts * stride * 2; q++) rf[q] = (float)rows[i][q];
        snprintf(path, sizeof(path), "%s/rows_i%d_s%d.c64", outdir, it, i);
        write_all(path, rf, (size_t)nffts * stride * 2 * sizeof(float));
        free(rf);
      }
      free(x);
      free(d.win);
    }
    int64_t(*nfl)[2] = xmalloc((size_t)nbl * sizeof(*nfl));
    find_invalid(&j, bl, nbl, w, nfl);
    if (j.phased) {
      /* Correlation_core_phased (sfxc/src/correlation_core_phased.cc): every
         FFT's spectra of all streams, in stream order, summed into the
         buffer of its sub-integration (current_fft / nsub); one "baseline"
         per buffer, headers from stream 0; no normalisation, no tsys */
      if (j.pulsar || j.n_pc > 1 || j.number_channels != M) die("phased array with pulsar / phase centres / reduction");
      const int nsubs = nffts / nsub + 1;
      double *acc = xmalloc((size_t)nsubs * K * 2 * sizeof(double));
      for (int r = 0; r < nffts; r++) {
        double *a = acc + (size_t)(r / nsub) * K * 2;
        for (int i = 0; i < j.nstreams; i++) {
          const double *x = rows[i] + (size_t)r * stride * 2;
          for (int k = 0; k < 2 * K; k++) a[k] = st(a[k] + x[k]);
        }
      }
      bl_t *pb = xmalloc((size_t)nsubs * sizeof(bl_t)); /* (0, 0) pairs */
      write_integration(&j, pb, nsubs, acc, w, nfl, nffts, it, 0, 0, &cor, &cor64);
      free(pb);
      free(acc);
    } else if (!j.pulsar) {
      double *acc = xmalloc((size_t)nbl * K * 2 * sizeof(double));
      double *pc = xmalloc((size_t)j.n_pc * nbl * K * 2 * sizeof(double)); /* phase_centers[c][b][k] */
      const size_t PCS = (size_t)nbl * K * 2;
      int cur = 0, next_sub = 1, prev = 0;
      const ticks_t tfft = (ticks_t)M * (ticks_t)(int)round(512000000.0 / j.sample_rate); /* Time(0, sr).inc_samples(M) */
      for (int c = 0; c < nchunks; c++) { /* Correlation_core::do_task per buffer (20-73) */
        xstep_rows(&j, bl, nbl, rows, stride, cur, cur + chunk[c], acc);
        cur += chunk[c];
        if (cur == nffts || cur >= next_sub * nsub) { /* sub_integration (516-559) */
          for (size_t q = 0; q < PCS; q++) pc[q] = st(pc[q] + acc[q]);
          if (j.n_pc > 1) {
            const ticks_t tmid = start + t_mul(tfft, prev + (cur - prev) / 2.);
            for (int c2 = 1; c2 < j.n_pc; c2++) {
              double *pcc = pc + c2 * PCS;
              for (size_t q = 0; q < (size_t)j.nstreams * K * 2; q++) pcc[q] = st(pcc[q] + acc[q]); /* autos */
              for (int b = j.nstreams; b < nbl; b++) {
                const int s1 = bl[b].a, s2 = bl[b].b;
                const double d1 = dt_delay(&ak[s1], tmid), d2 = dt_delay(&ak[s2], tmid);
                const double dd1 = dt_delay(&akp[s1 * j.n_pc + c2], tmid) - d1;
                const double dd2 = dt_delay(&akp[s2 * j.n_pc + c2], tmid) - d2;
                uvshift_add(&j, acc + (size_t)b * K * 2, pcc + (size_t)b * K * 2, dd1, dd2, dt_rate(&ak[s1], tmid),
                            dt_rate(&ak[s2], tmid));
              }
            }
          }
          for (size_t q = 0; q < PCS; q++) acc[q] = 0;
          prev = cur;
          if (cur != nffts) next_sub++;
        }
      }
      for (int c2 = 0; c2 < j.n_pc; c2++) {
        normalize(&j, bl, nbl, pc + c2 * PCS, w, nfl, nffts);
        write_integration(&j, bl, nbl, pc + c2 * PCS, w, nfl, nffts, it, j.pc_file[c2], c2, &cor, &cor64);
      }
      free(acc);
      free(pc);
    } else {
      /* Correlation_core_pulsar::set_parameters (13-99) */
      double us_per_day = (double)((int64_t)24 * 60 * 60 * 1000000);
      double start_mjd = t_get_mjd(start);
      double fft_duration = ((double)M * 1000000) / j.sample_rate;
      int closest = 0;
      double diff = fabs(j.polyco[0] - start_mjd);
      for (int p = 1; p < j.npolyco; p++) {
        double nd = fabs(j.polyco[p * 40] - start_mjd);
        if (nd < diff) {
          diff = nd;
          closest = p;
        }
      }
      const double *pc0 = j.polyco + closest * 40;
      double tmid = pc0[0], DM = pc0[1], ref_phase = pc0[2], ref_freq = pc0[3], obs_freq = pc0[4];
      int N = (int)pc0[5];
      const double *coef = pc0 + 6;
      /* The reference is built with -O2 -ffast-math (sfxc/configure.ac:31); GCC
         reassociates (start_mjd - tmid) + fft_duration/us_per_day into
         (start_mjd + fft_duration/us_per_day) - tmid.  Start MJDs carry ~6e-7 s
         of FP64 resolution, so the association moves the pulsar phase by up to
         ~1e-5 cycles; the compiled reference's order is restated here (checked
         against its own dumped start phase and bin table). */
      double DT;
      if (j.window == WINDOW_NONE)
        DT = ((start_mjd + fft_duration / (2 * us_per_day)) - tmid) * 1440;
      else
        DT = ((start_mjd + fft_duration / us_per_day) - tmid) * 1440;
      double start_phase = 0;
      for (int q = N - 1; q > 0; q--) start_phase = (start_phase + coef[q]) * DT;
      start_phase += (ref_phase - floor(ref_phase)) + DT * 60 * ref_freq + coef[0];
      int sb = j.sideband == 'L' ? -1 : 1;
      double base_freq = j.channel_freq * 1e-6;
      double dfreq = sb * j.sample_rate * 1e-6 / (2 * M);
      double inv_freq_obs2 = 1 / (obs_freq * obs_freq);
      double freq = 0;
      for (int q = N - 1; q > 1; q--) freq = (freq + q * coef[q]) * DT;
      freq = (freq + coef[1]) / 60 + ref_freq;
      double *offsets = xmalloc(K * 8);
      /* same build: 4148.808*DM*(...)*freq is evaluated as (4148.808*DM)*((...)*freq) */
      for (int q = 0; q < K; q++) {
        const double x = base_freq + q * dfreq;
        offsets[q] = (4148.808 * DM) * ((1 / (x * x) - inv_freq_obs2) * freq);
      }
      double len = j.gate1 - j.gate0;
      int nbins = j.nbins;
      double *acc = xmalloc((size_t)nbins * nbl * K * 2 * sizeof(double));
      int *bins = xmalloc(K * sizeof(int));
      FILE *binf = NULL;
      if (j.dump || j.dump_bins) {
        snprintf(path, sizeof(path), "%s/bins_i%d.i32", outdir, it);
        binf = fopen(path, "wb");
      }
      for (int r = 0; r < nffts; r++) { /* do_task + dedisperse_buffer (101-146, 210-238) */
        double obs_phase = start_phase + (coef[1] + 60 * ref_freq) * fft_duration * r * 1440 / us_per_day;
        for (int q = 0; q < K; q++) {
          double phase = obs_phase - offsets[q];
          phase = phase - floor(phase);
          if (phase >= j.gate0) {
            if (phase < j.gate1)
              bins[q] = (int)((phase - j.gate0) * (nbins - 1) / len) + 1;
            else
              bins[q] = 0;
          } else if (phase + 1 < j.gate1) {
            bins[q] = (int)((phase + 1 - j.gate0) * (nbins - 1) / len) + 1;
          } else {
            bins[q] = 0;
          }
        }
        if (binf) fwrite(bins, 4, K, binf);
        for (int b = 0; b < nbl; b++) {
          const double *x = rows[bl[b].a] + (size_t)r * stride * 2;
          const double *y = rows[bl[b].b] + (size_t)r * stride * 2;
          for (int q = 0; q < K; q++) {
            double *ac = acc + (((size_t)bins[q] * nbl + b) * K + q) * 2;
            double xr = x[2 * q], xi = x[2 * q + 1], yr = y[2 * q], yi = -y[2 * q + 1];
            if (g_f64) {
              ac[0] += xr * yr - xi * yi;
              ac[1] += xr * yi + xi * yr;
            } else {
              float pr = (float)((float)((float)xr * (float)yr) - (float)((float)xi * (float)yi));
              float pi = (float)((float)((float)xr * (float)yi) + (float)((float)xi * (float)yr));
              ac[0] = (float)((float)ac[0] + pr);
              ac[1] = (float)((float)ac[1] + pi);
            }
          }
        }
      }
      if (binf) fclose(binf);
      for (int bin = 0; bin < nbins; bin++) {
        double *a = acc + (size_t)bin * nbl * K * 2;
        normalize(&j, bl, nbl, a, w, nfl, nffts);
        write_integration(&j, bl, nbl, a, w, nfl, nffts, it, bin, 0, &cor, &cor64);
      }
      free(acc);
      free(bins);
      free(offsets);
    }
    if (!j.phased) tsys_write(&j, start, w, &tsys);
    for (int i = 0; i < j.nstreams; i++) {
      int lv[5], ts[4];
      stats_levels(&w[i].stats, lv);
      stats_tsys(&w[i].stats, ts);
      fprintf(statsf, "%d %d %d %d %d %d %d %d %d %d %d\n", it, lv[0], lv[1], lv[2], lv[3], lv[4], ts[0], ts[1],
              ts[2], ts[3], w[i].ninv);
      for (int q = 0; q < w[i].ninv; q++) fprintf(statsf, "I %d %d %d\n", i, w[i].inv[q].begin, w[i].inv[q].n);
    }
    for (int i = 0; i < j.nstreams; i++) {
      free(rows[i]);
      akima_free(&ak[i]);
      for (int c = 1; c < j.n_pc; c++) akima_free(&akp[i * j.n_pc + c]);
    }
    free(rows);
    free(ak);
    free(chunk);
    free(nfl);
  }
  fclose(statsf);
  snprintf(path, sizeof(path), "%s/out.cor", outdir);
  write_all(path, cor.p, cor.n);
  snprintf(path, sizeof(path), "%s/out64.bin", outdir);
  write_all(path, cor64.p, cor64.n);
  snprintf(path, sizeof(path), "%s/tsys.bin", outdir);
  write_all(path, tsys.p, tsys.n);
  return 0;
}

int main(int argc, char **argv) {
  if (argc != 4) die("usage: sfxc_oracle correlate|delays|protocol|extract <job> <out>");
  kvs_t k = read_job(argv[2]);
  if (!strcmp(argv[1], "correlate")) return mode_correlate(&k, argv[3]);
  if (!strcmp(argv[1], "delays")) return mode_delays(&k, argv[3]);
  if (!strcmp(argv[1], "protocol")) return mode_protocol(&k, argv[3]);
  if (!strcmp(argv[1], "extract")) return mode_extract(&k, argv[3]);
  die("unknown mode");
  return 2;
}
