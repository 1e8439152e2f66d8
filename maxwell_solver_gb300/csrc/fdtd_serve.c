/*
 * fdtd_serve.c -- the serving loop (fdtd_server_* in fdtd_gb300.h).
 *
 * One server thread owns all device work.  Clients submit requests (copied
 * into the queue) from any thread and wait on their tickets.  Each turn of
 * the loop:
 *   1. admits queued requests in arrival order while the sum of the
 *      admitted requests' peak device memory (fdtd_estimate_device_bytes)
 *      stays within the budget (and the active count within max_active);
 *      a request that can never fit fails at once, a request that does not
 *      fit yet holds the queue (no overtaking, so large solves are not
 *      starved);
 *   2. sets each admitted request up as an ordinary handle (SetParams,
 *      SetConst, SetShapes, SetAntennaLocations, ReadySimulation, Init1D):
 *      its fields, psi arrays and coefficients are resident from here on;
 *   3. picks the resident requests with the least remaining work (cells x
 *      steps left) until their cells reach the fill target that keeps the
 *      GPU busy, and advances those together with one fdtd_batch_step (at
 *      most round_steps steps; a round ends early when a member finishes);
 *      the others stay resident and wait -- shortest remaining work first,
 *      so small solves are not held back by large ones sharing the device;
 *      a round with a single request runs it with fdtd_step_n instead (the
 *      plain solver's graph-replayed kernels, for grids that fill the GPU
 *      alone);
 *   4. retires finished requests: outputs to host buffers, handle deleted,
 *      memory back to the budget, waiters woken.
 * Requests that arrive while others run are admitted at the next turn and
 * packed into the same batched launches -- continuous batching.  With
 * one_at_a_time set the loop instead takes one request at a time and runs
 * it to the end with fdtd_step_n: the plain-solver queue the batched form is
 * measured against.
 *
 * Every solve is the plain solver's arithmetic (the batched kernels give
 * results bit-identical to running alone), so a request's outputs do not
 * depend on what else was on the device.
 */
#include <errno.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/fdtd_gb300.h"
#include "fdtd_internal.h"

#define SFAIL(code, msg) fdtd_internal_fail((code), (msg))

#define MAX_SERVERS 64
#define ADMIT_MAX 64

typedef enum { R_QUEUED = 0, R_ACTIVE = 1, R_DONE = 2 } rstate;

typedef struct req {
  uint64_t ticket;
  fdtd_request r; /* its pointers point at the copies below */
  float *waveform;
  fdtd_shape *shapes;
  int32_t *probes;
  rstate state;
  fdtd_handle h;
  uint64_t est, held;
  double t_submit, t_admit, t_finish;
  int32_t status;
  char message[128];
  float *out_probes, *out_field;
  size_t n_out_probes, n_out_field;
  /* batched mode: stepping this round, steps completed before its current
   * stretch in the batch, and steps completed now */
  int in_batch, want;
  int cancel; /* fdtd_server_cancel while on the device (read with __atomic) */
  double key; /* this round's order (ascending) */
  double deadline; /* FDTD_SERVE_DEADLINE: finish time in a one-at-a-time queue */
  int32_t done_base, done;
  struct req *next;
} req;

/* phases of the serving loop (trace) */
enum { TR_SETUP, TR_SELECT, TR_SOLO, TR_BATCH, TR_PACE, TR_RETIRE, TR_N };
static const char *const k_tr_name[TR_N] = {"set-up", "select", "solo issue", "batch issue",
                                            "pacing wait", "retire"};

typedef struct server {
  fdtd_server_config cfg;
  pthread_t thread;
  int thread_started;
  pthread_mutex_t mu;
  pthread_cond_t cv_work, cv_done;
  int stop;
  struct timespec t0;
  /* ticket -> request (index ticket - 1; NULL once released) */
  req **tab;
  size_t tab_n, tab_cap;
  req *q_head, *q_tail;
  int queued, active; /* counts, under mu */
  uint64_t reserved;  /* sum of the active requests' peak estimates */
  /* server thread only: resident requests, and admitted ones (memory
   * reserved) whose set-up waits (deadline order, see serve_loop) */
  req **act;
  int n_act, cap_act;
  req **pend;
  int n_pend, cap_pend;
  fdtd_batch batch;
  /* pacing: an event after each round; the loop queues a round only once
   * the round before the last has finished, so that the order it picks
   * applies on the GPU within two rounds (nothing runs far ahead) */
  cudaEvent_t ev[2];
  int ev_used[2], ev_i;
  /* the one-at-a-time queue's estimated finish time of the last submission
   * (FDTD_SERVE_DEADLINE), under mu */
  double v_fifo;
  /* statistics, under mu */
  uint64_t submitted, completed, failed, cancelled, cell_steps, peak_reserved;
  int peak_active;
  double first_submit, last_finish;
  double *lat;
  size_t n_lat, cap_lat;
  /* server thread only: seconds and counts per phase of the loop, printed
   * to stderr at destroy when FDTD_SERVE_TRACE is set */
  double tr[TR_N];
  uint64_t trn[TR_N];
} server;

static pthread_mutex_t g_srv_lock = PTHREAD_MUTEX_INITIALIZER;
static server *g_srv[MAX_SERVERS];
static uint32_t g_srv_gen[MAX_SERVERS];

static server *slookup(fdtd_server h) {
  const uint32_t slot = (uint32_t)(h & 0xffffffffu), gen = (uint32_t)(h >> 32);
  if (slot == 0 || slot > MAX_SERVERS) return NULL;
  pthread_mutex_lock(&g_srv_lock);
  server *S = g_srv_gen[slot - 1] == gen ? g_srv[slot - 1] : NULL;
  pthread_mutex_unlock(&g_srv_lock);
  return S;
}

static double now_s(const server *S) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)(t.tv_sec - S->t0.tv_sec) + 1e-9 * (double)(t.tv_nsec - S->t0.tv_nsec);
}

static void free_req(req *r) {
  if (!r) return;
  free(r->waveform);
  free(r->shapes);
  free(r->probes);
  free(r->out_probes);
  free(r->out_field);
  free(r);
}

/* Marks r finished (status; msg NULL: the library's last error) and wakes
 * waiters; r may be released by a client as soon as this returns.  Server
 * thread. */
static void finish(server *S, req *r, int32_t status, const char *msg) {
  if (status != FDTD_OK) {
    snprintf(r->message, sizeof(r->message), "%s", msg ? msg : fdtd_last_error());
    free(r->out_probes);
    free(r->out_field);
    r->out_probes = r->out_field = NULL;
    r->n_out_probes = r->n_out_field = 0;
  }
  pthread_mutex_lock(&S->mu);
  r->status = status;
  r->t_finish = now_s(S);
  r->state = R_DONE;
  S->reserved -= r->est;
  S->active -= 1;
  if (status == FDTD_OK) {
    S->completed += 1;
    S->cell_steps += (uint64_t)r->r.I * r->r.J * r->r.K * (uint64_t)r->r.steps;
    if (S->n_lat == S->cap_lat) {
      const size_t nc = S->cap_lat ? 2 * S->cap_lat : 256;
      double *p = (double *)realloc(S->lat, nc * sizeof(double));
      if (p) {
        S->lat = p;
        S->cap_lat = nc;
      }
    }
    if (S->n_lat < S->cap_lat) S->lat[S->n_lat++] = r->t_finish - r->t_submit;
  } else if (status == FDTD_ERR_CANCELLED) {
    S->cancelled += 1;
  } else {
    S->failed += 1;
  }
  if (r->t_finish > S->last_finish) S->last_finish = r->t_finish;
  pthread_cond_broadcast(&S->cv_done);
  pthread_mutex_unlock(&S->mu);
}

/* The request as an ordinary handle, ready to step.  Server thread. */
static int setup(req *r) {
  const fdtd_request *q = &r->r;
  int rc = fdtd_create(&r->h);
  if (rc) return rc;
  const float fr[3] = {q->fctr, q->delX, q->delT};
  const int32_t td[5] = {q->steps, q->I, q->J, q->K, q->n_probes};
  if ((rc = fdtd_set_params(r->h, &q->params))) return rc;
  if ((rc = fdtd_set_const(r->h, fr, td))) return rc;
  if ((rc = fdtd_set_shapes(r->h, q->bg_eps_r, q->bg_sigma, r->shapes, q->n_shapes))) return rc;
  if (q->tfsf_mode == 5 && (rc = fdtd_set_incidence(r->h, q->theta, q->phi, q->psi))) return rc;
  if (q->n_probes > 0 &&
      (rc = fdtd_set_antenna_locations(r->h, r->probes, (size_t)q->n_probes * 3)))
    return rc;
  if ((rc = fdtd_ready_simulation(r->h))) return rc;
  if (q->tfsf_mode && (rc = fdtd_init_1d(r->h, q->rate, r->waveform, (size_t)q->steps)))
    return rc;
  fdtd_info info;
  if ((rc = fdtd_get_info(r->h, &info))) return rc;
  r->held = info.device_bytes;
  return FDTD_OK;
}

/* Outputs to the host, handle deleted.  Server thread. */
static int collect(server *S, req *r) {
  const fdtd_request *q = &r->r;
  int rc = FDTD_OK;
  if (q->n_probes > 0) {
    r->n_out_probes = (size_t)q->steps * q->n_probes * 6;
    r->out_probes = (float *)malloc(r->n_out_probes * sizeof(float));
    if (!r->out_probes) return FDTD_ERR_OOM;
    rc = fdtd_output_probes(r->h, r->out_probes, r->n_out_probes);
  }
  if (!rc && q->out_field >= 1 && q->out_field <= 6) {
    r->n_out_field = (size_t)q->I * q->J * q->K;
    r->out_field = (float *)malloc(r->n_out_field * sizeof(float));
    if (!r->out_field) return FDTD_ERR_OOM;
    rc = fdtd_output_vis(r->h, r->out_field, r->n_out_field, q->out_field);
  }
  if (!rc) rc = fdtd_synchronize(r->h);
  if (S->batch && r->in_batch) fdtd_batch_remove(S->batch, r->h);
  r->in_batch = 0;
  fdtd_destroy(r->h);
  r->h = 0;
  return rc;
}

/* (a handle that never joined the batch is not removed from it: that call
 * would fail and replace the message of the error being reported) */
static void drop_handle(server *S, req *r) {
  if (!r->h) return;
  if (S->batch && r->in_batch) fdtd_batch_remove(S->batch, r->h);
  r->in_batch = 0;
  fdtd_destroy(r->h);
  r->h = 0;
}

/* Every active request fails with rc (the batch is unusable). */
static void fail_active(server *S, int rc) {
  char m[128];
  snprintf(m, sizeof(m), "%s", fdtd_last_error());
  for (int a = 0; a < S->n_act; ++a) {
    drop_handle(S, S->act[a]);
    finish(S, S->act[a], rc, m);
  }
  S->n_act = 0;
  fdtd_batch_clear(S->batch);
}

static int64_t req_cells(const req *r) { return (int64_t)r->r.I * r->r.J * r->r.K; }

static int by_key(const void *a, const void *b) {
  const req *x = *(req *const *)a, *y = *(req *const *)b;
  return x->key < y->key ? -1 : x->key > y->key;
}

/* Approximate cell-steps per second of one GB300 on these kernels: the
 * scale between waiting time and remaining work in the response ratio. */
#define SERVE_RATE_EST 3.0e10
/* FDTD_SERVE_BOUNDED: the response ratio at which a request goes ahead
 * (3, or FDTD_SERVE_MAX_RATIO > 1; read once) */
static double serve_max_ratio(void) {
  static double v = 0.0;
  if (v <= 0.0) {
    const char *e = getenv("FDTD_SERVE_MAX_RATIO");
    const double x = e ? atof(e) : 0.0;
    v = x > 1.0 ? x : 3.0;
  }
  return v;
}

/* Estimated seconds a request of `cells` cells takes alone for `steps`
 * steps through fdtd_step_n (a fixed cost per step of the launches, then a
 * cell rate rising from 55 G cell-steps/s for small grids to 102 G at 100 M
 * cells), and its set-up with its readout (rasterising, indexing, a cached
 * autotune, the probe record).  Least-squares fit to the one-at-a-time
 * queue's service times of 100 mixed requests (0.1-55 M cells, 200-4000
 * steps) on GB300: within 6 % (standard deviation) per request, 1 % on
 * their sum. */
static double solo_step_s(int64_t cells) {
  const double c = (double)cells, rate = 5.55e10 + 4.66e10 * (c < 1.0e8 ? c / 1.0e8 : 1.0);
  return 2.7e-5 + c / rate;
}
static double solo_setup_s(int64_t cells) { return 3.0e-3 + (double)cells * 4.6e-10; }
/* Deadlines use those estimates times FDTD_SERVE_DEADLINE_SCALE (read
 * once; default 1.05: a request may finish up to about 5 % after its time
 * in the one-at-a-time queue, and that slack is what lets the smaller
 * requests go first).  At 1.0 the order stays near the queue's: the median
 * gain is gone while the tail still lands a few % above the queue's, since
 * both run the GPU at the same speed and estimate errors make the
 * deadline order miss by about that much; at 1.1 the median drops further
 * and the tail rises by up to a quarter under load. */
static double deadline_scale(void) {
  static double v = 0.0;
  if (v <= 0.0) {
    const char *e = getenv("FDTD_SERVE_DEADLINE_SCALE");
    const double x = e ? atof(e) : 0.0;
    v = x > 0.0 ? x : 1.05;
  }
  return v;
}
#define SERVE_DEADLINE_SCALE deadline_scale()
/* fdtd_step_n replays graphs of this many steps */
#define GRAPH_STEPS 32

static int by_deadline(const void *a, const void *b) {
  const req *x = *(req *const *)a, *y = *(req *const *)b;
  return x->deadline < y->deadline ? -1 : x->deadline > y->deadline;
}

/* Earliest deadline first over the resident requests: sorts S->act by
 * deadline and returns the last index of the urgent prefix (-1: none) --
 * if running them in that order would bring a request within the margin
 * of its deadline (the one-at-a-time queue's finish time), that request and
 * every one due before it are urgent. */
static int urgent_prefix(server *S, double now) {
  qsort(S->act, (size_t)S->n_act, sizeof(req *), by_deadline);
  double t = now;
  int last = -1;
  for (int a = 0; a < S->n_act; ++a) {
    req *r = S->act[a];
    const double left = SERVE_DEADLINE_SCALE * solo_step_s(req_cells(r)) * (r->r.steps - r->done);
    t += left;
    if (t + 0.15 * left + 0.1 > r->deadline) last = a;
  }
  return last;
}

static void order_requests(server *S, int policy) {
  const double now = now_s(S);
  for (int a = 0; a < S->n_act; ++a) {
    req *r = S->act[a];
    const double work = (double)req_cells(r) * (r->r.steps - r->done);
    const double rem = work / SERVE_RATE_EST + 1e-6;
    const double ratio = ((now - r->t_submit) + rem) / rem;
    if (policy == FDTD_SERVE_HRRN) {
      r->key = -ratio;
    } else if (policy == FDTD_SERVE_BOUNDED && ratio >= serve_max_ratio()) {
      r->key = -ratio; /* ahead of every key >= 0 below */
    } else {
      r->key = work;
    }
  }
  if (policy == FDTD_SERVE_DEADLINE && S->n_act > 1) {
    /* the urgent requests go ahead in deadline order; the others keep the
     * least-remaining-work order behind them */
    const int last = urgent_prefix(S, now);
    for (int a = 0; a <= last; ++a) S->act[a]->key = -1.0e12 + S->act[a]->deadline;
  }
  qsort(S->act, (size_t)S->n_act, sizeof(req *), by_key);
}

/* This round's members, in the policy's order (least remaining work,
 * highest response ratio, or least remaining work with the requests past
 * the ratio bound first).  When the first
 * request has at least `solo` cells it runs alone (*solo, through
 * fdtd_step_n, whose kernels are tuned to its shape); otherwise the smaller
 * requests are taken in order until their cells reach `fill`, and the large
 * ones wait.  Members that drop out leave the batch (their state stays
 * resident) and rejoin later at the step they reached.  A round of one
 * member also runs alone. */
static int select_round(server *S, int64_t fill, int64_t solo_cells, req **solo) {
  order_requests(S, S->cfg.policy);
  for (int a = 0; a < S->n_act; ++a) S->act[a]->want = 0;
  *solo = NULL;
  if (req_cells(S->act[0]) >= solo_cells) {
    *solo = S->act[0];
  } else {
    int n_want = 0;
    req *last = NULL;
    int64_t cells = 0;
    for (int a = 0; a < S->n_act && cells < fill; ++a) {
      req *r = S->act[a];
      if (req_cells(r) >= solo_cells) continue;
      r->want = 1;
      cells += req_cells(r);
      ++n_want;
      last = r;
    }
    if (n_want == 1) {
      *solo = last;
      last->want = 0;
    }
  }
  for (int a = 0; a < S->n_act; ++a) {
    req *r = S->act[a];
    const int want = r->want;
    int rc = FDTD_OK;
    if (want && !r->in_batch) {
      r->done_base = r->done;
      rc = fdtd_batch_add(S->batch, r->h, r->done, r->r.steps - r->done, r->r.tfsf_mode, NULL);
      r->in_batch = rc == FDTD_OK;
    } else if (!want && r->in_batch) {
      rc = fdtd_batch_remove(S->batch, r->h);
      r->in_batch = 0;
      r->done_base = r->done;
    }
    if (rc) return rc;
  }
  return FDTD_OK;
}

static void *serve_loop(void *arg) {
  server *S = (server *)arg;
  const int32_t round = S->cfg.round_steps > 0 ? S->cfg.round_steps : 32;
  const int64_t fill = S->cfg.fill_cells > 0 ? S->cfg.fill_cells : ((int64_t)1 << 25);
  const int64_t solo_cells = S->cfg.solo_cells > 0    ? S->cfg.solo_cells
                             : S->cfg.solo_cells == 0 ? ((int64_t)1 << 22)
                                                      : INT64_MAX;
  req *adm[ADMIT_MAX];
  pthread_mutex_lock(&S->mu);
  for (;;) {
    while (!S->stop && !S->q_head && S->n_act == 0 && S->n_pend == 0)
      pthread_cond_wait(&S->cv_work, &S->mu);
    if (S->stop && !S->q_head && S->n_act == 0 && S->n_pend == 0) break;
    /* 1. admission, in arrival order */
    int na = 0;
    while (S->q_head && na < ADMIT_MAX) {
      req *r = S->q_head;
      const int on_device = S->n_act + S->n_pend + na;
      if (S->cfg.one_at_a_time && on_device > 0) break;
      if (S->cfg.max_active > 0 && on_device >= S->cfg.max_active) break;
      const int never = r->est > S->cfg.hbm_budget;
      if (!never && S->reserved + r->est > S->cfg.hbm_budget) break;
      S->q_head = r->next;
      if (!S->q_head) S->q_tail = NULL;
      S->queued -= 1;
      S->active += 1;
      S->reserved += r->est;
      r->state = R_ACTIVE;
      r->t_admit = now_s(S);
      if (never) r->status = FDTD_ERR_OOM; /* finished below, outside the lock */
      adm[na++] = r;
    }
    if (S->reserved > S->peak_reserved) S->peak_reserved = S->reserved;
    if (S->active > S->peak_active) S->peak_active = S->active;
    pthread_mutex_unlock(&S->mu);

    /* 2. set-up (one at a time: set-up, every step, outputs).  In the
     * deadline order a set-up waits while a resident request is urgent: it
     * occupies the loop (and the GPU) for tens of ms, and a request that
     * arrived later is due later, so the urgent one goes first. */
    for (int a = 0; a < na; ++a) {
      req *r = adm[a];
      if (r->status == FDTD_ERR_OOM) {
        char m[128];
        snprintf(m, sizeof(m), "request needs %llu device bytes, budget %llu",
                 (unsigned long long)r->est, (unsigned long long)S->cfg.hbm_budget);
        finish(S, r, FDTD_ERR_OOM, m);
        continue;
      }
      if (S->n_pend == S->cap_pend) {
        const int nc = S->cap_pend ? 2 * S->cap_pend : 64;
        req **p = (req **)realloc(S->pend, (size_t)nc * sizeof(req *));
        if (!p) {
          finish(S, r, FDTD_ERR_OOM, "out of host memory");
          continue;
        }
        S->pend = p;
        S->cap_pend = nc;
      }
      S->pend[S->n_pend++] = r;
    }
    const int hold = S->cfg.policy == FDTD_SERVE_DEADLINE && !S->cfg.one_at_a_time &&
                     S->n_act > 0 && urgent_prefix(S, now_s(S)) >= 0;
    int kept = 0;
    for (int a = 0; a < S->n_pend; ++a) {
      req *r = S->pend[a];
      if (__atomic_load_n(&r->cancel, __ATOMIC_ACQUIRE)) { /* fdtd_server_cancel */
        finish(S, r, FDTD_ERR_CANCELLED, "cancelled");
        continue;
      }
      if (hold) {
        S->pend[kept++] = r;
        continue;
      }
      double t_ = now_s(S);
      int rc = setup(r);
      S->tr[TR_SETUP] += now_s(S) - t_;
      S->trn[TR_SETUP] += 1;
      if (!rc && S->cfg.one_at_a_time) {
        t_ = now_s(S);
        rc = fdtd_step_n(r->h, 0, r->r.steps, r->r.tfsf_mode, NULL);
        S->tr[TR_SOLO] += now_s(S) - t_;
        S->trn[TR_SOLO] += 1;
        t_ = now_s(S);
        if (!rc) rc = collect(S, r);
        S->tr[TR_RETIRE] += now_s(S) - t_;
        S->trn[TR_RETIRE] += 1;
        if (rc) drop_handle(S, r);
        finish(S, r, rc, NULL);
        continue;
      }
      if (rc) {
        drop_handle(S, r);
        finish(S, r, rc, NULL);
        continue;
      }
      if (S->n_act == S->cap_act) {
        const int nc = S->cap_act ? 2 * S->cap_act : 64;
        req **p = (req **)realloc(S->act, (size_t)nc * sizeof(req *));
        if (!p) {
          drop_handle(S, r);
          finish(S, r, FDTD_ERR_OOM, "out of host memory");
          continue;
        }
        S->act = p;
        S->cap_act = nc;
      }
      S->act[S->n_act++] = r;
    }
    S->n_pend = kept;

    /* 3. the round's members, then one round: the batch, or one request
     * alone through fdtd_step_n */
    req *solo = NULL;
    if (S->n_act > 0) {
      double t_ = now_s(S);
      int rc = select_round(S, fill, solo_cells, &solo);
      S->tr[TR_SELECT] += now_s(S) - t_;
      S->trn[TR_SELECT] += 1;
      t_ = now_s(S);
      if (!rc && solo) {
        /* a solo round lasts about 20 ms (at least `round` steps), so that
         * the loop's turn between rounds costs little next to it while a
         * request that must go ahead still waits at most one round */
        int32_t want = (int32_t)(0.02 / solo_step_s(req_cells(solo)));
        if (want < round) want = round;
        want = (want + GRAPH_STEPS - 1) / GRAPH_STEPS * GRAPH_STEPS;
        const int32_t n = solo->r.steps - solo->done < want ? solo->r.steps - solo->done : want;
        rc = fdtd_step_n(solo->h, solo->done, n, solo->r.tfsf_mode, NULL);
        if (!rc) solo->done_base = solo->done + n;
        else {
          drop_handle(S, solo);
          for (int a = 0; a < S->n_act; ++a)
            if (S->act[a] == solo) S->act[a] = S->act[--S->n_act];
          finish(S, solo, rc, NULL);
          solo = NULL;
          rc = FDTD_OK; /* only that request failed */
        }
      } else if (!rc) {
        int32_t left = 0;
        rc = fdtd_batch_step(S->batch, round, &left);
      }
      const int k_ = solo ? TR_SOLO : TR_BATCH;
      S->tr[k_] += now_s(S) - t_;
      S->trn[k_] += 1;
      t_ = now_s(S);
      if (!rc && S->ev[0]) { /* pace: wait for the previous round */
        const int e = solo ? fdtd_internal_record(solo->h, S->ev[S->ev_i])
                           : fdtd_internal_batch_record(S->batch, S->ev[S->ev_i]);
        S->ev_used[S->ev_i] = e == FDTD_OK;
        S->ev_i ^= 1;
        if (S->ev_used[S->ev_i]) {
          cudaEventSynchronize(S->ev[S->ev_i]);
          S->ev_used[S->ev_i] = 0;
        }
      }
      S->tr[TR_PACE] += now_s(S) - t_;
      S->trn[TR_PACE] += 1;
      if (rc) fail_active(S, rc);
    }
    const double t_ret = now_s(S);

    /* 4. retire the finished ones (after checking the batch's pipelines
     * completed: a bounded wait that timed out invalidates the round) */
    int any = 0;
    for (int a = 0; a < S->n_act; ++a) {
      req *r = S->act[a];
      int32_t p = 0;
      if (r->in_batch) fdtd_batch_progress(S->batch, r->h, &p);
      r->done = r->done_base + (p > 0 ? p : 0);
      any |= r->done >= r->r.steps;
    }
    if (any) {
      const int rc = fdtd_batch_status(S->batch);
      if (rc) fail_active(S, rc);
    }
    for (int a = 0; a < S->n_act;) {
      req *r = S->act[a];
      if (__atomic_load_n(&r->cancel, __ATOMIC_ACQUIRE)) { /* fdtd_server_cancel */
        drop_handle(S, r);
        finish(S, r, FDTD_ERR_CANCELLED, "cancelled");
        S->act[a] = S->act[--S->n_act];
        continue;
      }
      if (r->done < r->r.steps) {
        ++a;
        continue;
      }
      const int rc = collect(S, r);
      if (rc) drop_handle(S, r);
      finish(S, r, rc, NULL);
      S->act[a] = S->act[--S->n_act];
      S->trn[TR_RETIRE] += 1;
    }
    S->tr[TR_RETIRE] += now_s(S) - t_ret;
    pthread_mutex_lock(&S->mu);
  }
  pthread_mutex_unlock(&S->mu);
  return NULL;
}

static void release_gpu(server *S) {
  if (S->batch) fdtd_batch_destroy(S->batch);
  S->batch = 0;
  for (int i = 0; i < 2; ++i)
    if (S->ev[i]) cudaEventDestroy(S->ev[i]);
}

int fdtd_server_create(fdtd_server *out, const fdtd_server_config *cfg) {
  if (!out || !cfg) return FDTD_ERR_INVALID_ARG;
  if (cfg->policy != FDTD_SERVE_SRPT && cfg->policy != FDTD_SERVE_HRRN &&
      cfg->policy != FDTD_SERVE_BOUNDED && cfg->policy != FDTD_SERVE_DEADLINE)
    return FDTD_ERR_INVALID_ARG;
  server *S = (server *)calloc(1, sizeof(server));
  if (!S) return FDTD_ERR_OOM;
  S->cfg = *cfg;
  if (!S->cfg.hbm_budget) { /* admit by the device memory free now */
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      free(S);
      return FDTD_ERR_CUDA;
    }
    S->cfg.hbm_budget = (uint64_t)((double)free_b * 0.9);
  }
  clock_gettime(CLOCK_MONOTONIC, &S->t0);
  S->first_submit = -1.0;
  pthread_mutex_init(&S->mu, NULL);
  pthread_condattr_t ca;
  pthread_condattr_init(&ca);
  pthread_condattr_setclock(&ca, CLOCK_MONOTONIC);
  pthread_cond_init(&S->cv_work, &ca);
  pthread_cond_init(&S->cv_done, &ca);
  pthread_condattr_destroy(&ca);
  int rc = FDTD_OK;
  if (!cfg->one_at_a_time) {
    rc = fdtd_batch_create(&S->batch);
    for (int i = 0; i < 2 && !rc; ++i)
      if (cudaEventCreateWithFlags(&S->ev[i], cudaEventDisableTiming) != cudaSuccess)
        rc = FDTD_ERR_CUDA;
  }
  if (!rc && pthread_create(&S->thread, NULL, serve_loop, S) != 0) rc = FDTD_ERR_OOM;
  if (rc) {
    release_gpu(S);
    free(S);
    return rc;
  }
  S->thread_started = 1;
  pthread_mutex_lock(&g_srv_lock);
  int slot = -1;
  for (int i = 0; i < MAX_SERVERS; ++i)
    if (!g_srv[i]) {
      slot = i;
      break;
    }
  if (slot >= 0) {
    g_srv[slot] = S;
    g_srv_gen[slot] += 1;
    *out = ((uint64_t)g_srv_gen[slot] << 32) | (uint64_t)(slot + 1);
  }
  pthread_mutex_unlock(&g_srv_lock);
  if (slot < 0) {
    pthread_mutex_lock(&S->mu);
    S->stop = 1;
    pthread_cond_broadcast(&S->cv_work);
    pthread_mutex_unlock(&S->mu);
    pthread_join(S->thread, NULL);
    release_gpu(S);
    free(S);
    return FDTD_ERR_OOM;
  }
  return FDTD_OK;
}

int fdtd_server_submit(fdtd_server h, const fdtd_request *q, uint64_t *ticket) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  if (!q || !ticket || q->steps < 1 || q->n_shapes < 0 || q->n_probes < 0 ||
      (q->tfsf_mode && !q->waveform) || (q->n_shapes && !q->shapes) ||
      (q->n_probes && !q->probes))
    return SFAIL(FDTD_ERR_INVALID_ARG, "request: steps >= 1 and the arrays its counts name");
  req *r = (req *)calloc(1, sizeof(req));
  if (!r) return FDTD_ERR_OOM;
  r->r = *q;
  int rc = fdtd_estimate_device_bytes(q->I, q->J, q->K, q->params.pml, q->steps, q->n_probes,
                                      &r->est);
  if (!rc && q->tfsf_mode) {
    r->waveform = (float *)malloc((size_t)q->steps * sizeof(float));
    if (!r->waveform) rc = FDTD_ERR_OOM;
    else memcpy(r->waveform, q->waveform, (size_t)q->steps * sizeof(float));
  }
  if (!rc) {
    r->shapes = (fdtd_shape *)malloc((size_t)(q->n_shapes ? q->n_shapes : 1) * sizeof(fdtd_shape));
    if (!r->shapes) rc = FDTD_ERR_OOM;
    else if (q->n_shapes) memcpy(r->shapes, q->shapes, (size_t)q->n_shapes * sizeof(fdtd_shape));
  }
  if (!rc && q->n_probes) {
    r->probes = (int32_t *)malloc((size_t)q->n_probes * 3 * sizeof(int32_t));
    if (!r->probes) rc = FDTD_ERR_OOM;
    else memcpy(r->probes, q->probes, (size_t)q->n_probes * 3 * sizeof(int32_t));
  }
  if (rc) {
    free_req(r);
    return rc;
  }
  r->r.waveform = r->waveform;
  r->r.shapes = r->shapes;
  r->r.probes = r->probes;
  pthread_mutex_lock(&S->mu);
  if (S->tab_n == S->tab_cap) {
    const size_t nc = S->tab_cap ? 2 * S->tab_cap : 256;
    req **p = (req **)realloc(S->tab, nc * sizeof(req *));
    if (!p) {
      pthread_mutex_unlock(&S->mu);
      free_req(r);
      return FDTD_ERR_OOM;
    }
    S->tab = p;
    S->tab_cap = nc;
  }
  S->tab[S->tab_n] = r;
  r->ticket = ++S->tab_n;
  r->t_submit = now_s(S);
  if (S->first_submit < 0) S->first_submit = r->t_submit;
  { /* the one-at-a-time queue: starts when it arrives or the one before ends */
    const int64_t cells = (int64_t)q->I * q->J * q->K;
    const double start = S->v_fifo > r->t_submit ? S->v_fifo : r->t_submit;
    S->v_fifo = start + SERVE_DEADLINE_SCALE * (solo_setup_s(cells) + solo_step_s(cells) * q->steps);
    r->deadline = S->v_fifo;
  }
  r->state = R_QUEUED;
  if (S->q_tail) S->q_tail->next = r;
  else S->q_head = r;
  S->q_tail = r;
  S->queued += 1;
  S->submitted += 1;
  *ticket = r->ticket;
  pthread_cond_broadcast(&S->cv_work);
  pthread_mutex_unlock(&S->mu);
  return FDTD_OK;
}

static req *ticket_req(server *S, uint64_t t) {
  return (t >= 1 && t <= S->tab_n) ? S->tab[t - 1] : NULL;
}

int fdtd_server_wait(fdtd_server h, uint64_t ticket, double timeout_s) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  struct timespec dl;
  clock_gettime(CLOCK_MONOTONIC, &dl);
  if (timeout_s >= 0) {
    const double t = (double)dl.tv_sec + 1e-9 * (double)dl.tv_nsec + timeout_s;
    dl.tv_sec = (time_t)t;
    dl.tv_nsec = (long)((t - (double)dl.tv_sec) * 1e9);
  }
  pthread_mutex_lock(&S->mu);
  req *r = ticket_req(S, ticket);
  int rc = FDTD_OK;
  while (r && r->state != R_DONE) {
    if (timeout_s < 0) {
      pthread_cond_wait(&S->cv_done, &S->mu);
    } else if (pthread_cond_timedwait(&S->cv_done, &S->mu, &dl) == ETIMEDOUT) {
      rc = FDTD_ERR_STATE;
      break;
    }
    r = ticket_req(S, ticket);
  }
  if (!r) rc = FDTD_ERR_INVALID_ARG;
  pthread_mutex_unlock(&S->mu);
  return rc;
}

int fdtd_server_result(fdtd_server h, uint64_t ticket, float *probes, size_t n_probes,
                       float *field, size_t n_field, fdtd_request_info *info) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  pthread_mutex_lock(&S->mu);
  req *r = ticket_req(S, ticket);
  if (!r || r->state != R_DONE) {
    pthread_mutex_unlock(&S->mu);
    return r ? FDTD_ERR_STATE : FDTD_ERR_INVALID_ARG;
  }
  S->tab[ticket - 1] = NULL;
  pthread_mutex_unlock(&S->mu);
  if (probes && r->out_probes)
    memcpy(probes, r->out_probes,
           (n_probes < r->n_out_probes ? n_probes : r->n_out_probes) * sizeof(float));
  if (field && r->out_field)
    memcpy(field, r->out_field,
           (n_field < r->n_out_field ? n_field : r->n_out_field) * sizeof(float));
  if (info) {
    snprintf(info->message, sizeof(info->message), "%s", r->message);
    info->submit_s = r->t_submit;
    info->admit_s = r->t_admit;
    info->finish_s = r->t_finish;
    info->device_bytes = r->held;
    info->status = r->status;
    info->steps = r->r.steps;
  }
  const int32_t st = r->status;
  free_req(r);
  return st;
}

int fdtd_server_cancel(fdtd_server h, uint64_t ticket) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  pthread_mutex_lock(&S->mu);
  req *r = ticket_req(S, ticket);
  int rc = FDTD_OK;
  if (!r) {
    rc = SFAIL(FDTD_ERR_INVALID_ARG, "unknown or released ticket");
  } else if (r->state == R_DONE) {
    rc = SFAIL(FDTD_ERR_STATE, "the request has already finished");
  } else if (r->state == R_QUEUED) { /* out of the queue, finished now */
    req *prev = NULL;
    for (req *q = S->q_head; q; prev = q, q = q->next)
      if (q == r) {
        if (prev) prev->next = r->next;
        else S->q_head = r->next;
        if (S->q_tail == r) S->q_tail = prev;
        break;
      }
    r->next = NULL;
    S->queued -= 1;
    snprintf(r->message, sizeof(r->message), "cancelled");
    r->status = FDTD_ERR_CANCELLED;
    r->t_finish = now_s(S);
    r->state = R_DONE;
    S->cancelled += 1;
    pthread_cond_broadcast(&S->cv_done);
  } else { /* on the device: the loop drops it at the end of the round */
    __atomic_store_n(&r->cancel, 1, __ATOMIC_RELEASE);
  }
  pthread_mutex_unlock(&S->mu);
  return rc;
}

int fdtd_server_drain(fdtd_server h) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  pthread_mutex_lock(&S->mu);
  while (S->queued > 0 || S->active > 0) pthread_cond_wait(&S->cv_done, &S->mu);
  pthread_mutex_unlock(&S->mu);
  return FDTD_OK;
}

static int cmp_double(const void *a, const void *b) {
  const double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : x > y;
}

/* Nearest-rank percentile of sorted values. */
static double pct(const double *v, size_t n, double p) {
  if (!n) return 0.0;
  size_t k = (size_t)(p / 100.0 * (double)n + 0.999999999);
  if (k < 1) k = 1;
  if (k > n) k = n;
  return v[k - 1];
}

int fdtd_server_get_stats(fdtd_server h, fdtd_server_stats *out) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  if (!out) return FDTD_ERR_INVALID_ARG;
  memset(out, 0, sizeof(*out));
  pthread_mutex_lock(&S->mu);
  out->submitted = S->submitted;
  out->completed = S->completed;
  out->failed = S->failed;
  out->cancelled = S->cancelled;
  out->cell_steps = S->cell_steps;
  out->peak_reserved_bytes = S->peak_reserved;
  out->peak_active = S->peak_active;
  out->queued = S->queued;
  out->active = S->active;
  out->hbm_budget = S->cfg.hbm_budget;
  out->elapsed_s = S->first_submit >= 0 && S->last_finish > S->first_submit
                       ? S->last_finish - S->first_submit
                       : 0.0;
  const size_t n = S->n_lat;
  double *v = n ? (double *)malloc(n * sizeof(double)) : NULL;
  if (v) memcpy(v, S->lat, n * sizeof(double));
  pthread_mutex_unlock(&S->mu);
  if (v) {
    qsort(v, n, sizeof(double), cmp_double);
    double sum = 0.0;
    for (size_t i = 0; i < n; ++i) sum += v[i];
    out->latency_mean_s = sum / (double)n;
    out->latency_p50_s = pct(v, n, 50.0);
    out->latency_p90_s = pct(v, n, 90.0);
    out->latency_p99_s = pct(v, n, 99.0);
    free(v);
  }
  out->solves_per_s = out->elapsed_s > 0 ? (double)out->completed / out->elapsed_s : 0.0;
  return FDTD_OK;
}

int fdtd_server_destroy(fdtd_server h) {
  server *S = slookup(h);
  if (!S) return SFAIL(FDTD_ERR_INVALID_HANDLE, "invalid server handle");
  fdtd_server_drain(h);
  pthread_mutex_lock(&g_srv_lock);
  const uint32_t slot = (uint32_t)(h & 0xffffffffu);
  g_srv[slot - 1] = NULL;
  pthread_mutex_unlock(&g_srv_lock);
  pthread_mutex_lock(&S->mu);
  S->stop = 1;
  pthread_cond_broadcast(&S->cv_work);
  pthread_mutex_unlock(&S->mu);
  if (S->thread_started) pthread_join(S->thread, NULL);
  if (getenv("FDTD_SERVE_TRACE")) {
    fprintf(stderr, "fdtd serve trace (%s, %llu completed, %.3f s first submission to last result):\n",
            S->cfg.one_at_a_time ? "one at a time" : "served", (unsigned long long)S->completed,
            S->last_finish - S->first_submit);
    for (int k = 0; k < TR_N; ++k)
      fprintf(stderr, "  %-12s %9.3f s  %8llu\n", k_tr_name[k], S->tr[k],
              (unsigned long long)S->trn[k]);
    uint64_t n[2] = {0, 0};
    double t[2] = {0, 0};
    if (S->batch && fdtd_internal_batch_counts(S->batch, n, t) == FDTD_OK)
      fprintf(stderr, "  batch rebuilds %llu (%.3f s), graph captures %llu (%.3f s)\n",
              (unsigned long long)n[0], t[0], (unsigned long long)n[1], t[1]);
  }
  release_gpu(S);
  for (size_t i = 0; i < S->tab_n; ++i) free_req(S->tab[i]);
  free(S->tab);
  free(S->act);
  free(S->pend);
  free(S->lat);
  pthread_cond_destroy(&S->cv_work);
  pthread_cond_destroy(&S->cv_done);
  pthread_mutex_destroy(&S->mu);
  free(S);
  return FDTD_OK;
}
