/*
 * gbode_oracle.c -- CPU oracle for the adaptive embedded Runge-Kutta N-body
 * path.  TEST INFRASTRUCTURE ONLY: the GPU library never links, loads or
 * calls anything in this file.  It is imported by the tests, by the smoke
 * check and by the CPU-baseline leg of bench.py, always as the oracle the GPU
 * results are compared against (or as the timed reference CPU implementation),
 * never as the product.
 *
 * It is a plain-C restatement of the reference's algorithm, operation for
 * operation, so that with one thread it reproduces the reference's
 * single-threaded executor bit for bit (the parity tests pin it against the
 * reference's own golden values and against the reference compiled in place).
 * With several threads it mirrors the reference's spin-waiting thread pool:
 * a static block partition of the items, double atomic adds implemented as
 * compare-and-swap loops, and per-thread partial sums for the reduction.
 *
 * Reference files restated here (paths inside noether17/ode_prototyping):
 *   src/integrator/RKEmbeddedParallel/RKEmbeddedParallel.hpp:13-200
 *   src/integrator/RKEmbeddedParallel/butcher_tableaus/BT*.hpp
 *   src/ode/NBodyODE.hpp:31-133, src/ode/ExponentialODE.hpp:10-18,
 *   src/ode/VanDerPolODE.hpp:12-25
 *   src/par_exec/SingleThreadedExecutor.hpp:7-30,
 *   src/par_exec/ThreadPoolExecutor.hpp:12-114, src/util/AtomicUtil.hpp:7-12
 *   src/integrator/leapfrog/LeapfrogParallel.hpp:11-73
 *   scripts/nbody_physics/energy.py:146-192 (softened potential energy)
 *
 * Build: cc -O2 -std=c11 -ffp-contract=off -fno-fast-math -fPIC -shared
 *        -pthread (oracle/Makefile).  -ffp-contract=off keeps a*b+c as two
 *        roundings on every host (the reference's x86-64 build has no FMA).
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAX_STAGES 16

typedef struct {
  int n_stages;
  int p;
  int pt;
  double a[ORC_MAX_STAGES][ORC_MAX_STAGES]; /* a[stage-1][j], j < stage */
  double b[ORC_MAX_STAGES];
  double bt[ORC_MAX_STAGES];
} orc_tableau;

enum { ORC_HE21 = 0, ORC_RKF45 = 1, ORC_DOPRI5 = 2, ORC_DVERK = 3, ORC_RKF78 = 4 };

/* Butcher tableaus, butcher_tableaus/BT{HE21,RKF45,DOPRI5,DVERK,RKF78}.hpp.
 * The coefficients are the published rational values; the compiler folds
 * each quotient to the nearest double exactly as the reference's constexpr
 * arrays do. */
int orc_tableau_builtin(int id, orc_tableau* t) {
  memset(t, 0, sizeof *t);
#define A(r, c, v) t->a[r][c] = (v)
  switch (id) {
    case ORC_HE21: /* BTHE21.hpp:5-12 */
      t->n_stages = 2; t->p = 2; t->pt = 1;
      A(0, 0, 1.0);
      t->b[0] = 1.0 / 2.0; t->b[1] = 1.0 / 2.0;
      t->bt[0] = 1.0; t->bt[1] = 0.0;
      return 0;
    case ORC_RKF45: /* BTRKF45.hpp:5-21 */
      t->n_stages = 6; t->p = 4; t->pt = 5;
      A(0, 0, 1.0 / 4.0);
      A(1, 0, 3.0 / 32.0); A(1, 1, 9.0 / 32.0);
      A(2, 0, 1932.0 / 2197.0); A(2, 1, -7200.0 / 2197.0); A(2, 2, 7296.0 / 2197.0);
      A(3, 0, 439.0 / 216.0); A(3, 1, -8.0); A(3, 2, 3680.0 / 513.0); A(3, 3, -845.0 / 4104.0);
      A(4, 0, -8.0 / 27.0); A(4, 1, 2.0); A(4, 2, -3544.0 / 2565.0); A(4, 3, 1859.0 / 4104.0);
      A(4, 4, -11.0 / 40.0);
      t->b[0] = 25.0 / 216.0; t->b[2] = 1408.0 / 2565.0; t->b[3] = 2197.0 / 4104.0; t->b[4] = -0.2;
      t->bt[0] = 16.0 / 135.0; t->bt[2] = 6656.0 / 12825.0; t->bt[3] = 28561.0 / 56430.0;
      t->bt[4] = -9.0 / 50.0; t->bt[5] = 2.0 / 55.0;
      return 0;
    case ORC_DOPRI5: /* BTDOPRI5.hpp:5-26 */
      t->n_stages = 7; t->p = 5; t->pt = 4;
      A(0, 0, 1.0 / 5.0);
      A(1, 0, 3.0 / 40.0); A(1, 1, 9.0 / 40.0);
      A(2, 0, 44.0 / 45.0); A(2, 1, -56.0 / 15.0); A(2, 2, 32.0 / 9.0);
      A(3, 0, 19372.0 / 6561.0); A(3, 1, -25360.0 / 2187.0); A(3, 2, 64448.0 / 6561.0);
      A(3, 3, -212.0 / 729.0);
      A(4, 0, 9017.0 / 3168.0); A(4, 1, -355.0 / 33.0); A(4, 2, 46732.0 / 5247.0);
      A(4, 3, 49.0 / 176.0); A(4, 4, -5103.0 / 18656.0);
      A(5, 0, 35.0 / 384.0); A(5, 2, 500.0 / 1113.0); A(5, 3, 125.0 / 192.0);
      A(5, 4, -2187.0 / 6784.0); A(5, 5, 11.0 / 84.0);
      t->b[0] = 35.0 / 384.0; t->b[2] = 500.0 / 1113.0; t->b[3] = 125.0 / 192.0;
      t->b[4] = -2187.0 / 6784.0; t->b[5] = 11.0 / 84.0;
      t->bt[0] = 5179.0 / 57600.0; t->bt[2] = 7571.0 / 16695.0; t->bt[3] = 393.0 / 640.0;
      t->bt[4] = -92097.0 / 339200.0; t->bt[5] = 187.0 / 2100.0; t->bt[6] = 1.0 / 40.0;
      return 0;
    case ORC_DVERK: /* BTDVERK.hpp:5-27 */
      t->n_stages = 8; t->p = 6; t->pt = 5;
      A(0, 0, 1.0 / 6.0);
      A(1, 0, 4.0 / 75.0); A(1, 1, 16.0 / 75.0);
      A(2, 0, 5.0 / 6.0); A(2, 1, -8.0 / 3.0); A(2, 2, 5.0 / 2.0);
      A(3, 0, -165.0 / 64.0); A(3, 1, 55.0 / 6.0); A(3, 2, -425.0 / 64.0); A(3, 3, 85.0 / 96.0);
      A(4, 0, 12.0 / 5.0); A(4, 1, -8.0); A(4, 2, 4015.0 / 612.0); A(4, 3, -11.0 / 36.0);
      A(4, 4, 88.0 / 255.0);
      A(5, 0, -8263.0 / 15000.0); A(5, 1, 124.0 / 75.0); A(5, 2, -643.0 / 680.0);
      A(5, 3, -81.0 / 250.0); A(5, 4, 2484.0 / 10625.0);
      A(6, 0, 3501.0 / 1720.0); A(6, 1, -300.0 / 43.0); A(6, 2, 297275.0 / 52632.0);
      A(6, 3, -319.0 / 2322.0); A(6, 4, 24068.0 / 84065.0); A(6, 6, 3850.0 / 26703.0);
      t->b[0] = 3.0 / 40.0; t->b[2] = 875.0 / 2244.0; t->b[3] = 23.0 / 72.0;
      t->b[4] = 264.0 / 1955.0; t->b[6] = 125.0 / 11592.0; t->b[7] = 43.0 / 616.0;
      t->bt[0] = 13.0 / 160.0; t->bt[2] = 2375.0 / 5984.0; t->bt[3] = 5.0 / 16.0;
      t->bt[4] = 12.0 / 85.0; t->bt[5] = 3.0 / 44.0;
      return 0;
    case ORC_RKF78: /* BTRKF78.hpp:5-45 */
      t->n_stages = 13; t->p = 7; t->pt = 8;
      A(0, 0, 2.0 / 27.0);
      A(1, 0, 1.0 / 36.0); A(1, 1, 1.0 / 12.0);
      A(2, 0, 1.0 / 24.0); A(2, 2, 1.0 / 8.0);
      A(3, 0, 5.0 / 12.0); A(3, 2, -25.0 / 16.0); A(3, 3, 25.0 / 16.0);
      A(4, 0, 1.0 / 20.0); A(4, 3, 1.0 / 4.0); A(4, 4, 1.0 / 5.0);
      A(5, 0, -25.0 / 108.0); A(5, 3, 125.0 / 108.0); A(5, 4, -65.0 / 27.0); A(5, 5, 125.0 / 54.0);
      A(6, 0, 31.0 / 300.0); A(6, 4, 61.0 / 225.0); A(6, 5, -2.0 / 9.0); A(6, 6, 13.0 / 900.0);
      A(7, 0, 2.0); A(7, 3, -53.0 / 6.0); A(7, 4, 704.0 / 45.0); A(7, 5, -107.0 / 9.0);
      A(7, 6, 67.0 / 90.0); A(7, 7, 3.0);
      A(8, 0, -91.0 / 108.0); A(8, 3, 23.0 / 108.0); A(8, 4, -976.0 / 135.0);
      A(8, 5, 311.0 / 54.0); A(8, 6, -19.0 / 60.0); A(8, 7, 17.0 / 6.0); A(8, 8, -1.0 / 12.0);
      A(9, 0, 2383.0 / 4100.0); A(9, 3, -341.0 / 164.0); A(9, 4, 4496.0 / 1025.0);
      A(9, 5, -301.0 / 82.0); A(9, 6, 2133.0 / 4100.0); A(9, 7, 45.0 / 82.0);
      A(9, 8, 45.0 / 164.0); A(9, 9, 18.0 / 41.0);
      A(10, 0, 3.0 / 205.0); A(10, 5, -6.0 / 41.0); A(10, 6, -3.0 / 205.0);
      A(10, 7, -3.0 / 41.0); A(10, 8, 3.0 / 41.0); A(10, 9, 6.0 / 41.0);
      A(11, 0, -1777.0 / 4100.0); A(11, 3, -341.0 / 164.0); A(11, 4, 4496.0 / 1025.0);
      A(11, 5, -289.0 / 82.0); A(11, 6, 2193.0 / 4100.0); A(11, 7, 51.0 / 82.0);
      A(11, 8, 33.0 / 164.0); A(11, 9, 12.0 / 41.0); A(11, 11, 1.0);
      t->b[0] = 41.0 / 840.0; t->b[5] = 34.0 / 105.0; t->b[6] = 9.0 / 35.0;
      t->b[7] = 9.0 / 35.0; t->b[8] = 9.0 / 280.0; t->b[9] = 9.0 / 280.0; t->b[10] = 41.0 / 840.0;
      t->bt[5] = 34.0 / 105.0; t->bt[6] = 9.0 / 35.0; t->bt[7] = 9.0 / 35.0;
      t->bt[8] = 9.0 / 280.0; t->bt[9] = 9.0 / 280.0; t->bt[11] = 41.0 / 840.0;
      t->bt[12] = 41.0 / 840.0;
      return 0;
    default:
      return -1;
  }
#undef A
}

/* ------------------------------------------------------------------------ */
/* Thread pool mirroring ThreadPoolExecutor.hpp:26-124: workers spin on a   */
/* per-thread ready flag (yielding every 8 polls, :12-24), take the static  */
/* block [id*ceil(n/T), min((id+1)*ceil(n/T), n)) of the items (:42-49) and */
/* count a latch down; the caller waits on the latch (:62-79).              */
/* ------------------------------------------------------------------------ */
typedef void (*orc_task_fn)(void* ctx, int64_t begin, int64_t end, int thread_id);

typedef struct {
  int n_threads;
  pthread_t* threads;
  volatile int* ready; /* per-thread flags */
  volatile int stop;
  volatile int64_t n_items;
  orc_task_fn fn;
  void* ctx;
  int64_t latch;
} orc_pool;

typedef struct {
  orc_pool* pool;
  int id;
} orc_worker_arg;

static int orc_spin_until_ready(orc_pool* p, int id) {
  for (int trial = 0; !__atomic_load_n(&p->stop, __ATOMIC_ACQUIRE); ++trial) {
    if (__atomic_load_n(&p->ready[id], __ATOMIC_ACQUIRE)) return 1;
    if (trial == 8) {
      trial = 0;
      sched_yield();
    }
  }
  return 0;
}

static void* orc_worker(void* argp) {
  orc_worker_arg* arg = (orc_worker_arg*)argp;
  orc_pool* p = arg->pool;
  int id = arg->id;
  free(arg);
  for (;;) {
    if (!orc_spin_until_ready(p, id)) return NULL;
    __atomic_store_n(&p->ready[id], 0, __ATOMIC_RELEASE);
    int64_t n = __atomic_load_n(&p->n_items, __ATOMIC_ACQUIRE);
    int64_t per = (n + p->n_threads - 1) / p->n_threads;
    int64_t b = id * per;
    int64_t e = (id + 1) * per < n ? (id + 1) * per : n;
    if (b < e) p->fn(p->ctx, b, e, id);
    __atomic_sub_fetch(&p->latch, 1, __ATOMIC_ACQ_REL);
  }
}

static orc_pool* orc_pool_create(int n_threads) {
  orc_pool* p = (orc_pool*)calloc(1, sizeof *p);
  p->n_threads = n_threads;
  p->threads = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
  p->ready = (volatile int*)calloc((size_t)n_threads, sizeof(int));
  for (int i = 0; i < n_threads; ++i) {
    orc_worker_arg* a = (orc_worker_arg*)malloc(sizeof *a);
    a->pool = p;
    a->id = i;
    pthread_create(&p->threads[i], NULL, orc_worker, a);
  }
  return p;
}

static void orc_pool_destroy(orc_pool* p) {
  if (!p) return;
  __atomic_store_n(&p->stop, 1, __ATOMIC_RELEASE);
  for (int i = 0; i < p->n_threads; ++i) pthread_join(p->threads[i], NULL);
  free(p->threads);
  free((void*)p->ready);
  free(p);
}

static void orc_pool_run(orc_pool* p, int64_t n_items, orc_task_fn fn, void* ctx) {
  p->fn = fn;
  p->ctx = ctx;
  __atomic_store_n(&p->n_items, n_items, __ATOMIC_RELEASE);
  __atomic_store_n(&p->latch, (int64_t)p->n_threads, __ATOMIC_RELEASE);
  for (int i = 0; i < p->n_threads; ++i) __atomic_store_n(&p->ready[i], 1, __ATOMIC_RELEASE);
  int trial = 0;
  while (__atomic_load_n(&p->latch, __ATOMIC_ACQUIRE) != 0) {
    if (++trial == 8) {
      trial = 0;
      sched_yield();
    }
  }
}

/* Executor: NULL pool = SingleThreadedExecutor (serial loop over i). */
static void orc_exec(orc_pool* p, int64_t n, orc_task_fn fn, void* ctx) {
  if (!p) {
    if (n > 0) fn(ctx, 0, n, 0);
  } else {
    orc_pool_run(p, n, fn, ctx);
  }
}

/* au::atomic_add (AtomicUtil.hpp:7-12): std::atomic_ref<double> += b is a
 * compare-and-swap loop on the bit pattern. */
static inline void orc_atomic_add(double* target, double v) {
  uint64_t* bits = (uint64_t*)target;
  uint64_t expected = __atomic_load_n(bits, __ATOMIC_RELAXED);
  for (;;) {
    double cur;
    memcpy(&cur, &expected, sizeof cur);
    double next = cur + v;
    uint64_t desired;
    memcpy(&desired, &next, sizeof desired);
    if (__atomic_compare_exchange_n(bits, &expected, desired, 1, __ATOMIC_SEQ_CST,
                                    __ATOMIC_RELAXED))
      return;
  }
}

/* ------------------------------------------------------------------------ */
/* ODEs                                                                      */
/* ------------------------------------------------------------------------ */
enum { ORC_ODE_NBODY = 0, ORC_ODE_EXPONENTIAL = 1, ORC_ODE_VANDERPOL = 2 };

typedef struct {
  int64_t n_particles;
  double softening;      /* NBodyODE::softening (NBodyODE.hpp:29) */
  double mass;           /* uniform mass applied after the pair sum (0 => 1) */
  const double* masses;  /* per-body masses (the masses.size()>1 branch of
                            NBodyODE.hpp:104-124); NULL => uniform mass */
} orc_nbody;

typedef struct {
  int kind;
  orc_nbody nb;
  int64_t n_var;
} orc_ode;

typedef struct {
  const orc_nbody* nb;
  const double* pos;
  double* acc;
  double eps2;
  int use_atomics;
} orc_pair_ctx;

/* nbody_acc_kernel (NBodyODE.hpp:68-133): one item per unordered pair,
 * (i, j) recovered from the pair id with a double square root. */
static void orc_pair_task(void* vctx, int64_t begin, int64_t end, int tid) {
  (void)tid;
  orc_pair_ctx* c = (orc_pair_ctx*)vctx;
  const uint64_t n = (uint64_t)c->nb->n_particles;
  const double* pos = c->pos;
  double* acc = c->acc;
  const double* m = c->nb->masses;
  for (int64_t pid = begin; pid < end; ++pid) {
    uint64_t pair_id = (uint64_t)pid;
    double n_minus_half = (double)n - 0.5;
    uint64_t i =
        (uint64_t)(n_minus_half - sqrt(n_minus_half * n_minus_half - 2.0 * (double)pair_id));
    uint64_t j = pair_id - (n - 1) * i + (i * (i + 1)) / 2 + 1;
    double dx = pos[3 * j] - pos[3 * i];
    double dy = pos[3 * j + 1] - pos[3 * i + 1];
    double dz = pos[3 * j + 2] - pos[3 * i + 2];
    double dist_sq = dx * dx + dy * dy + dz * dz + c->eps2;
    double dist = sqrt(dist_sq);
    double den = dist * dist_sq;
    double ax = dx / den, ay = dy / den, az = dz / den;
    double axi = ax, ayi = ay, azi = az;
    double axj = -ax, ayj = -ay, azj = -az;
    if (m) {
      axi *= m[j]; ayi *= m[j]; azi *= m[j];
      axj *= m[i]; ayj *= m[i]; azj *= m[i];
    }
    if (c->use_atomics) {
      orc_atomic_add(&acc[3 * i], axi);
      orc_atomic_add(&acc[3 * i + 1], ayi);
      orc_atomic_add(&acc[3 * i + 2], azi);
      orc_atomic_add(&acc[3 * j], axj);
      orc_atomic_add(&acc[3 * j + 1], ayj);
      orc_atomic_add(&acc[3 * j + 2], azj);
    } else {
      acc[3 * i] += axi;
      acc[3 * i + 1] += ayi;
      acc[3 * i + 2] += azi;
      acc[3 * j] += axj;
      acc[3 * j + 1] += ayj;
      acc[3 * j + 2] += azj;
    }
  }
}

typedef struct {
  const double* x;
  double* dxdt;
  int64_t n_dof;
  double scale;
} orc_init_ctx;

/* nbody_init_dxdt_kernel (NBodyODE.hpp:51-56). */
static void orc_init_dxdt_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_init_ctx* c = (orc_init_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) {
    c->dxdt[i] = c->x[i + c->n_dof];
    c->dxdt[i + c->n_dof] = 0.0;
  }
}

/* Uniform-mass scaling of the acceleration half, applied after the pair sum. */
static void orc_scale_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_init_ctx* c = (orc_init_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) c->dxdt[i + c->n_dof] *= c->scale;
}

static void orc_nbody_eval(orc_pool* pool, const orc_nbody* nb, const double* x, double* dxdt) {
  const int64_t n = nb->n_particles;
  const int64_t n_dof = 3 * n;
  orc_init_ctx ic = {x, dxdt, n_dof, 1.0};
  orc_exec(pool, n_dof, orc_init_dxdt_task, &ic);
  orc_pair_ctx pc = {nb, x, dxdt + n_dof, nb->softening * nb->softening, pool != NULL};
  orc_exec(pool, n * (n - 1) / 2, orc_pair_task, &pc);
  if (!nb->masses && nb->mass != 0.0 && nb->mass != 1.0) {
    ic.scale = nb->mass;
    orc_exec(pool, n_dof, orc_scale_task, &ic);
  }
}

typedef struct {
  const double* x;
  double* dxdt;
} orc_simple_ctx;

static void orc_expo_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_simple_ctx* c = (orc_simple_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) c->dxdt[i] = c->x[i]; /* ExponentialODE.hpp:15-18 */
}

static void orc_vdp_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_simple_ctx* c = (orc_simple_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) { /* VanDerPolODE.hpp:17-25, mu = 1 */
    if (i == 0) {
      c->dxdt[0] = c->x[1];
    } else if (i == 1) {
      const double eps = 1.0;
      c->dxdt[1] = eps * (1.0 - c->x[0] * c->x[0]) * c->x[1] - c->x[0];
    }
  }
}

static void orc_ode_eval(orc_pool* pool, const orc_ode* ode, const double* x, double* dxdt) {
  orc_simple_ctx sc = {x, dxdt};
  switch (ode->kind) {
    case ORC_ODE_NBODY: orc_nbody_eval(pool, &ode->nb, x, dxdt); break;
    case ORC_ODE_EXPONENTIAL: orc_exec(pool, ode->n_var, orc_expo_task, &sc); break;
    case ORC_ODE_VANDERPOL: orc_exec(pool, 2, orc_vdp_task, &sc); break;
    default: break;
  }
}

/* ------------------------------------------------------------------------ */
/* Element-wise RK kernels (RKEmbeddedParallel.hpp:91-168)                  */
/* ------------------------------------------------------------------------ */
typedef struct {
  const orc_tableau* bt;
  int stage;
  double dt;
  double* temp;
  const double* ks;
  const double* x0;
  double* x;
  double* err;
  double* target;
  const double* atol;
  const double* rtol;
  int64_t n_var;
  double db[ORC_MAX_STAGES];
} orc_rk_ctx;

/* rk_stage_kernel (:91-101): accumulate from 0.0, j ascending, then x0 + s*dt. */
static void orc_stage_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_rk_ctx* c = (orc_rk_ctx*)vctx;
  const int s = c->stage;
  for (int64_t i = b; i < e; ++i) {
    double v = 0.0;
    for (int j = 0; j < s; ++j) v += c->bt->a[s - 1][j] * c->ks[j * c->n_var + i];
    c->temp[i] = c->x0[i] + v * c->dt;
  }
}

/* update_state_and_error_kernel (:103-123), db = b - bt folded beforehand. */
static void orc_update_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_rk_ctx* c = (orc_rk_ctx*)vctx;
  const int S = c->bt->n_stages;
  for (int64_t i = b; i < e; ++i) {
    double xv = 0.0, ev = 0.0;
    for (int j = 0; j < S; ++j) {
      xv += c->bt->b[j] * c->ks[j * c->n_var + i];
      ev += c->db[j] * c->ks[j * c->n_var + i];
    }
    c->x[i] = c->x0[i] + xv * c->dt;
    c->err[i] = ev * c->dt;
  }
}

/* update_error_target_kernel (:125-130): new and old state. */
static void orc_target_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_rk_ctx* c = (orc_rk_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) {
    double ax = fabs(c->x[i]), ax0 = fabs(c->x0[i]);
    c->target[i] = c->atol[i] + c->rtol[i] * (ax < ax0 ? ax0 : ax);
  }
}

/* compute_error_target_kernel (:151-156). */
static void orc_target0_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_rk_ctx* c = (orc_rk_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) c->target[i] = fabs(c->x0[i]) * c->rtol[i] + c->atol[i];
}

/* euler_step_kernel (:158-162): x1 = x0 + f0*dt0 (temp <- x0 + ks*dt). */
static void orc_euler_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_rk_ctx* c = (orc_rk_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) c->temp[i] = c->x0[i] + c->ks[i] * c->dt;
}

/* difference_kernel (:164-167): df -= f0 (err <- err - ks). */
static void orc_diff_task(void* vctx, int64_t b, int64_t e, int tid) {
  (void)tid;
  orc_rk_ctx* c = (orc_rk_ctx*)vctx;
  for (int64_t i = b; i < e; ++i) c->err[i] -= c->ks[i];
}

typedef struct {
  const double* v;
  const double* scale;
  int64_t n;
  int64_t per_thread;
  double* partials;
} orc_norm_ctx;

/* ThreadPoolExecutor::transform_reduce_kernel (:81-97): thread t sums the
 * block [t*per, min((t+1)*per, n)) from T{} = 0.0. */
static void orc_norm_partial_task(void* vctx, int64_t b, int64_t e, int tid) {
  orc_norm_ctx* c = (orc_norm_ctx*)vctx;
  (void)e;
  int64_t t = b; /* one item per thread */
  (void)tid;
  double acc = 0.0;
  for (int64_t i = t * c->per_thread; i < (t + 1) * c->per_thread && i < c->n; ++i) {
    double s = c->v[i] / c->scale[i];
    acc = acc + s * s;
  }
  c->partials[t] = acc;
}

/* rk_norm (:141-149): sqrt(transform_reduce(0.0, n, (v/scale)^2) / n). */
static double orc_rk_norm(orc_pool* pool, const double* v, const double* scale, int64_t n) {
  double sum;
  if (!pool) { /* SingleThreadedExecutor.hpp:17-28 */
    sum = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      double s = v[i] / scale[i];
      sum = sum + s * s;
    }
  } else { /* ThreadPoolExecutor.hpp:99-114 */
    int T = pool->n_threads;
    double partials[256];
    double* parts = T <= 256 ? partials : (double*)malloc((size_t)T * sizeof(double));
    orc_norm_ctx nc = {v, scale, n, (n + T - 1) / T, parts};
    orc_pool_run(pool, T, orc_norm_partial_task, &nc);
    sum = 0.0;
    for (int t = 0; t < T; ++t) sum = sum + parts[t];
    if (parts != partials) free(parts);
  }
  return sqrt(sum / (double)n);
}

/* ------------------------------------------------------------------------ */
/* Integrator (RKEmbeddedParallel.hpp:13-81, estimate_initial_step 170-200) */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t n_saved;     /* accepted steps + 1 */
  int64_t n_attempts;
  int64_t n_rejected;
  int64_t n_rhs;
  double dt_initial;
  double t_final;
  int status;          /* 0 ok, 1 output capacity exceeded, 2 attempt limit */
} orc_stats;

/* Saved-state sink: times[k], states[k*n_var ...] for k < capacity.  When
 * keep_every_state == 0 only the latest state is kept (in states[0]). */
typedef struct {
  double* times;
  double* states;
  int64_t capacity;
  int keep_all;
} orc_sink;

static void orc_save(orc_sink* s, orc_stats* st, double t, const double* x, int64_t n_var) {
  int64_t k = st->n_saved++;
  if (s->keep_all) {
    if (k < s->capacity) {
      if (s->times) s->times[k] = t;
      if (s->states) memcpy(s->states + k * n_var, x, (size_t)n_var * sizeof(double));
    } else {
      st->status = 1;
    }
  } else {
    if (s->times) s->times[0] = t;
    if (s->states) memcpy(s->states, x, (size_t)n_var * sizeof(double));
  }
}

static double orc_estimate_initial_step(orc_pool* pool, const orc_tableau* bt,
                                        const orc_ode* ode, const double* x0,
                                        const double* atol, const double* rtol,
                                        int64_t n_var, orc_stats* st) {
  double* target = (double*)malloc((size_t)n_var * sizeof(double));
  double* f0 = (double*)malloc((size_t)n_var * sizeof(double));
  double* x1 = (double*)malloc((size_t)n_var * sizeof(double));
  double* df = (double*)malloc((size_t)n_var * sizeof(double));
  orc_rk_ctx c;
  memset(&c, 0, sizeof c);
  c.bt = bt;
  c.n_var = n_var;
  c.x0 = x0;
  c.atol = atol;
  c.rtol = rtol;
  c.target = target;
  orc_exec(pool, n_var, orc_target0_task, &c);
  orc_ode_eval(pool, ode, x0, f0);
  st->n_rhs++;
  double d0 = orc_rk_norm(pool, x0, target, n_var);
  double d1 = orc_rk_norm(pool, f0, target, n_var);
  double dt0 = (d0 < 1.0e-5 || d1 < 1.0e-5) ? 1.0e-6 : 0.01 * (d0 / d1);
  c.temp = x1;
  c.ks = f0;
  c.dt = dt0;
  orc_exec(pool, n_var, orc_euler_task, &c);
  orc_ode_eval(pool, ode, x1, df);
  st->n_rhs++;
  c.err = df;
  orc_exec(pool, n_var, orc_diff_task, &c);
  double d2 = orc_rk_norm(pool, df, target, n_var) / dt0;
  double dmax = d1 < d2 ? d2 : d1;
  double dt1;
  if (dmax <= 1.0e-15) {
    double alt = dt0 * 1.0e-3;
    dt1 = alt < 1.0e-6 ? 1.0e-6 : alt;
  } else {
    dt1 = pow(0.01 / dmax, 1.0 / (1.0 + bt->p));
  }
  free(target);
  free(f0);
  free(x1);
  free(df);
  double big = 100.0 * dt0;
  return dt1 < big ? dt1 : big;
}

/* PI step-size controller, restating NumericalRecipes/StepperDopr5.hpp:
 * 236-272 (Controller::success) with its constants as parameters: on an
 * accepted step scale = safe * err^-alpha * errold^beta (maxscale when
 * err == 0), clamped to [minscale, maxscale], no increase right after a
 * rejection, errold = max(err, 1e-4); a rejection scales by
 * max(safe * err^-alpha, minscale).  Returns the factor applied to h. */
typedef struct {
  double safe, alpha, beta, minscale, maxscale, errold;
  int reject;
} orc_pi;

static double orc_pi_scale(orc_pi* c, double err, int accepted) {
  double scale;
  if (accepted) {
    if (err == 0.0) {
      scale = c->maxscale;
    } else {
      scale = c->safe * pow(err, -c->alpha) * pow(c->errold, c->beta);
      if (scale < c->minscale) scale = c->minscale;
      if (scale > c->maxscale) scale = c->maxscale;
    }
    if (c->reject && scale > 1.0) scale = 1.0;
    c->errold = err > 1.0e-4 ? err : 1.0e-4;
    c->reject = 0;
  } else {
    scale = c->safe * pow(err, -c->alpha);
    if (scale < c->minscale) scale = c->minscale;
    c->reject = 1;
  }
  return scale;
}

/* Resumable form of the reference's adaptive loop: a session holds the
 * loop state (t, dt, x0, buffers, executor) of RKEmbeddedParallel::integrate
 * so that attempts can be run and timed one at a time. */
typedef struct {
  orc_tableau bt;
  orc_ode ode;
  orc_pool* pool;
  int64_t n_var;
  double t0, tf, t, dt, safety_factor;
  int q;
  double *x0, *x, *ks, *temp, *err, *target, *atol, *rtol;
  orc_rk_ctx c;
  orc_stats st;
  /* step-size controller: 0 = the reference's elementary controller
   * (RKEmbeddedParallel.hpp:65-74), 1 = PI (orc_pi_step) */
  int controller;
  orc_pi pi;
  /* DOPRI5 dense output: outputs at dense_t[0..n_dense) (ascending) into
   * dense_out[j * n_var ...]; dense_next = first output not yet produced */
  const double* dense_t;
  double* dense_out;
  int64_t n_dense, dense_next;
} orc_session;

/* The controller alone on a sequence of error norms (accepted iff err <= 1,
 * as in Controller::success), starting from step h0: hs[k] = the step after
 * the k-th decision (hnext on success, the reduced h on a rejection).  Used
 * to pin orc_pi_scale to the reference's own Controller::success. */
int orc_pi_sequence(double safe, double alpha, double beta, double minscale, double maxscale,
                    const double* errs, int64_t n, double h0, double* hs) {
  if (!errs || !hs || n < 0) return -1;
  orc_pi c = {safe, alpha, beta, minscale, maxscale, 1.0e-4, 0};
  double h = h0;
  for (int64_t k = 0; k < n; ++k) {
    const double scale = orc_pi_scale(&c, errs[k], errs[k] <= 1.0);
    h = h * scale;
    hs[k] = h;
  }
  return 0;
}

/* The session's PI controller (GB_CTRL_PI on the GPU): orc_pi_scale with
 * the reference integrator's constants instead of Numerical Recipes' (safe =
 * 0.38^(1/(1+q)), minscale 0.33, maxscale 6, RKEmbeddedParallel.hpp:21-24;
 * alpha = 1/(1+q) - 0.75 beta), and the reference's floor on the new step
 * at (tf - t0) * 1e-12 (:71-72). */
static double orc_pi_step(orc_session* ss, double dt, double err, int accepted) {
  double dtn = dt * orc_pi_scale(&ss->pi, err, accepted);
  if (dtn / (ss->tf - ss->t0) < 1.0e-12) dtn = (ss->tf - ss->t0) * 1.0e-12;
  return dtn;
}

/* DOPRI5 dense output over the step just accepted (y0 at t_old, y1 at
 * t_old + h), restating NumericalRecipes/StepperDopr5.hpp:179-219:
 * prepare_dense's rcont1..5 from y0, y1 and the stage derivatives k1, k3..k7
 * (k7 = f(y1), the seventh stage), then dense_out's polynomial in
 * s = (t - (t_new - h)) / h. */
static void orc_dopri5_dense(const double* y0, const double* y1, const double* ks, int64_t n,
                             double h, double t_new, const double* ts, int64_t nt,
                             double* out) {
  const double d1 = -12715105075.0 / 11282082432.0, d3 = 87487479700.0 / 32700410799.0,
               d4 = -10690763975.0 / 1880347072.0, d5 = 701980252875.0 / 199316789632.0,
               d6 = -1453857185.0 / 822651844.0, d7 = 69997945.0 / 29380423.0;
  const double *k1 = ks, *k3 = ks + 2 * n, *k4 = ks + 3 * n, *k5 = ks + 4 * n,
               *k6 = ks + 5 * n, *k7 = ks + 6 * n;
  for (int64_t i = 0; i < n; ++i) {
    const double r1 = y0[i];
    const double ydiff = y1[i] - y0[i];
    const double r2 = ydiff;
    const double bspl = h * k1[i] - ydiff;
    const double r3 = bspl;
    const double r4 = ydiff - h * k7[i] - bspl;
    const double r5 =
        h * (d1 * k1[i] + d3 * k3[i] + d4 * k4[i] + d5 * k5[i] + d6 * k6[i] + d7 * k7[i]);
    for (int64_t j = 0; j < nt; ++j) {
      const double sv = (ts[j] - (t_new - h)) / h;
      const double s1 = 1.0 - sv;
      out[j * n + i] = r1 + sv * (r2 + s1 * (r3 + sv * (r4 + s1 * r5)));
    }
  }
}

orc_session* orc_session_create(const orc_tableau* bt, const orc_ode* ode, const double* x0_in,
                                double t0, double tf, const double* atol, const double* rtol,
                                int n_threads) {
  if (!bt || !ode || !x0_in || !atol || !rtol || bt->n_stages < 1 ||
      bt->n_stages > ORC_MAX_STAGES)
    return NULL;
  orc_session* ss = (orc_session*)calloc(1, sizeof *ss);
  ss->bt = *bt;
  ss->ode = *ode;
  const int64_t n_var = ode->n_var;
  const int S = bt->n_stages;
  ss->n_var = n_var;
  ss->t0 = t0;
  ss->tf = tf;
  ss->q = bt->p < bt->pt ? bt->p : bt->pt;
  ss->safety_factor = pow(0.38, (1.0 / (1.0 + ss->q)));
  ss->pool = n_threads > 1 ? orc_pool_create(n_threads) : NULL;
  size_t vb = (size_t)n_var * sizeof(double);
  ss->x0 = (double*)malloc(vb);
  ss->x = (double*)malloc(vb);
  ss->ks = (double*)malloc(vb * (size_t)S);
  ss->temp = (double*)calloc((size_t)n_var, sizeof(double));
  ss->err = (double*)calloc((size_t)n_var, sizeof(double));
  ss->target = (double*)calloc((size_t)n_var, sizeof(double));
  ss->atol = (double*)malloc(vb);
  ss->rtol = (double*)malloc(vb);
  memcpy(ss->x0, x0_in, vb);
  memcpy(ss->atol, atol, vb);
  memcpy(ss->rtol, rtol, vb);
  ss->dt = orc_estimate_initial_step(ss->pool, &ss->bt, &ss->ode, ss->x0, ss->atol, ss->rtol,
                                     n_var, &ss->st);
  ss->st.dt_initial = ss->dt;
  ss->t = t0;
  memcpy(ss->x, ss->x0, vb);
  orc_rk_ctx* c = &ss->c;
  c->bt = &ss->bt;
  c->n_var = n_var;
  c->ks = ss->ks;
  c->x0 = ss->x0;
  c->x = ss->x;
  c->temp = ss->temp;
  c->err = ss->err;
  c->target = ss->target;
  c->atol = ss->atol;
  c->rtol = ss->rtol;
  for (int j = 0; j < S; ++j) c->db[j] = bt->b[j] - bt->bt[j];
  return ss;
}

/* One attempt of the loop body (RKEmbeddedParallel.hpp:36-79).  Returns 1
 * when the loop condition t < tf no longer holds (nothing done), else 0;
 * *accepted reports the decision. */
int orc_session_attempt(orc_session* ss, int* accepted) {
  if (!(ss->t < ss->tf)) return 1;
  orc_pool* pool = ss->pool;
  const int S = ss->bt.n_stages;
  const int64_t n_var = ss->n_var;
  orc_rk_ctx* c = &ss->c;
  ss->st.n_attempts++;
  c->dt = ss->dt;
  orc_ode_eval(pool, &ss->ode, ss->x0, ss->ks);
  for (int stage = 1; stage < S; ++stage) {
    c->stage = stage;
    orc_exec(pool, n_var, orc_stage_task, c);
    orc_ode_eval(pool, &ss->ode, ss->temp, ss->ks + (int64_t)stage * n_var);
  }
  ss->st.n_rhs += S;
  orc_exec(pool, n_var, orc_update_task, c);
  orc_exec(pool, n_var, orc_target_task, c);
  double scaled_error = orc_rk_norm(pool, ss->err, ss->target, n_var);
  double dt = ss->dt;
  int acc = scaled_error <= 1.0;
  if (acc) {
    ss->t += dt;
    if (ss->dense_out && S == 7) {
      int64_t j1 = ss->dense_next;
      while (j1 < ss->n_dense && ss->dense_t[j1] <= ss->t) ++j1;
      if (j1 > ss->dense_next)
        orc_dopri5_dense(ss->x0, ss->x, ss->ks, n_var, dt, ss->t, ss->dense_t + ss->dense_next,
                         j1 - ss->dense_next, ss->dense_out + ss->dense_next * n_var);
      ss->dense_next = j1;
    }
    memcpy(ss->x0, ss->x, (size_t)n_var * sizeof(double));
  } else {
    ss->st.n_rejected++;
  }
  if (ss->controller == 1) {
    dt = orc_pi_step(ss, dt, scaled_error, acc);
  } else {
    double dtnew = dt * ss->safety_factor / pow(scaled_error, 1.0 / (1.0 + ss->q));
    if (fabs(dtnew) > 6.0 * fabs(dt)) {
      dt *= 6.0;
    } else if (fabs(dtnew) < 0.33 * fabs(dt)) {
      dt *= 0.33;
    } else if (dtnew / (ss->tf - ss->t0) < 1.0e-12) {
      dt = (ss->tf - ss->t0) * 1.0e-12;
    } else {
      dt = dtnew;
    }
  }
  if (ss->t + dt > ss->tf) dt = ss->tf - ss->t;
  ss->dt = dt;
  ss->st.t_final = ss->t;
  if (accepted) *accepted = acc;
  return 0;
}

/* The dense formula alone (for pinning it to the reference's own
 * prepare_dense / dense_out): ks holds the seven stage derivatives
 * stage-major (ks[j * n + i]). */
int orc_dopri5_dense_eval(const double* y0, const double* y1, const double* ks, int64_t n,
                          double h, double t_new, const double* ts, int64_t nt, double* out) {
  if (!y0 || !y1 || !ks || !ts || !out || n < 0 || nt < 0 || !(h != 0.0)) return -1;
  orc_dopri5_dense(y0, y1, ks, n, h, t_new, ts, nt, out);
  return 0;
}

/* Switches the session's step-size controller: kind 0 = the reference's
 * elementary controller, 1 = PI with the given beta (alpha = 1/(1+q) -
 * 0.75 beta, errold starting at 1e-4).  Call before the first attempt. */
int orc_session_set_controller(orc_session* ss, int kind, double beta) {
  if (!ss || (kind != 0 && kind != 1)) return -1;
  ss->controller = kind;
  orc_pi c = {ss->safety_factor, 1.0 / (1.0 + ss->q) - 0.75 * beta, beta, 0.33, 6.0, 1.0e-4, 0};
  ss->pi = c;
  return 0;
}

/* DOPRI5 dense output at the ascending times ts[0..nt) into out[nt][n_var]
 * (caller-owned, kept alive while the session runs).  Returns -1 unless the
 * session's tableau has seven stages (DOPRI5). */
int orc_session_set_dense(orc_session* ss, const double* ts, int64_t nt, double* out) {
  if (!ss || ss->bt.n_stages != 7 || nt < 0 || (nt > 0 && (!ts || !out))) return -1;
  ss->dense_t = ts;
  ss->dense_out = out;
  ss->n_dense = nt;
  ss->dense_next = 0;
  return 0;
}

/* Number of dense outputs produced so far. */
int64_t orc_session_dense_count(const orc_session* ss) { return ss ? ss->dense_next : 0; }

const double* orc_session_state(const orc_session* ss, double* t) {
  if (t) *t = ss->t;
  return ss->x0;
}

void orc_session_stats(const orc_session* ss, orc_stats* st) { *st = ss->st; }

void orc_session_destroy(orc_session* ss) {
  if (!ss) return;
  orc_pool_destroy(ss->pool);
  free(ss->x0);
  free(ss->x);
  free(ss->ks);
  free(ss->temp);
  free(ss->err);
  free(ss->target);
  free(ss->atol);
  free(ss->rtol);
  free(ss);
}

/* Integrates x' = f(x) from t0 to tf with the reference's adaptive loop.
 * n_threads <= 1 runs the single-threaded executor; otherwise a thread pool
 * of n_threads.  max_attempts > 0 bounds the loop (status 2 when hit; the
 * reference itself has no bound).  Returns 0, or -1 on a bad argument. */
int orc_rk_integrate(const orc_tableau* bt, const orc_ode* ode, const double* x0_in, double t0,
                     double tf, const double* atol, const double* rtol, int n_threads,
                     int64_t max_attempts, double* times, double* states, int64_t capacity,
                     int keep_all, orc_stats* st) {
  if (!st) return -1;
  orc_session* ss = orc_session_create(bt, ode, x0_in, t0, tf, atol, rtol, n_threads);
  if (!ss) return -1;
  orc_sink sink = {times, states, capacity, keep_all};
  orc_stats* sst = &ss->st;
  int status = 0;
  orc_save(&sink, sst, ss->t, ss->x0, ss->n_var);
  while (ss->t < tf) {
    if (max_attempts > 0 && sst->n_attempts >= max_attempts) {
      status = 2;
      break;
    }
    int acc = 0;
    orc_session_attempt(ss, &acc);
    if (acc) orc_save(&sink, sst, ss->t, ss->x0, ss->n_var);
  }
  if (status) sst->status = status;
  sst->t_final = ss->t;
  *st = *sst;
  orc_session_destroy(ss);
  return 0;
}

/* One fixed-step embedded RK step (no acceptance test): x1 = x0 + dt*sum b k,
 * err = dt*sum (b-bt) k, and the scaled norm -- the building blocks above in
 * the reference's order.  Used for fixed-step trajectory parity. */
int orc_rk_fixed_steps(const orc_tableau* bt, const orc_ode* ode, double* x_inout, double dt,
                       int64_t n_steps, const double* atol, const double* rtol, int n_threads,
                       double* err_norms) {
  if (!bt || !ode || !x_inout) return -1;
  const int64_t n_var = ode->n_var;
  const int S = bt->n_stages;
  orc_pool* pool = n_threads > 1 ? orc_pool_create(n_threads) : NULL;
  double* x0 = (double*)malloc((size_t)n_var * sizeof(double));
  double* ks = (double*)malloc((size_t)n_var * (size_t)S * sizeof(double));
  double* temp = (double*)calloc((size_t)n_var, sizeof(double));
  double* err = (double*)calloc((size_t)n_var, sizeof(double));
  double* target = (double*)calloc((size_t)n_var, sizeof(double));
  memcpy(x0, x_inout, (size_t)n_var * sizeof(double));
  orc_rk_ctx c;
  memset(&c, 0, sizeof c);
  c.bt = bt;
  c.n_var = n_var;
  c.ks = ks;
  c.x0 = x0;
  c.x = x_inout;
  c.temp = temp;
  c.err = err;
  c.target = target;
  c.atol = atol;
  c.rtol = rtol;
  c.dt = dt;
  for (int j = 0; j < S; ++j) c.db[j] = bt->b[j] - bt->bt[j];
  for (int64_t step = 0; step < n_steps; ++step) {
    orc_ode_eval(pool, ode, x0, ks);
    for (int stage = 1; stage < S; ++stage) {
      c.stage = stage;
      orc_exec(pool, n_var, orc_stage_task, &c);
      orc_ode_eval(pool, ode, temp, ks + (int64_t)stage * n_var);
    }
    orc_exec(pool, n_var, orc_update_task, &c);
    if (atol && rtol) {
      orc_exec(pool, n_var, orc_target_task, &c);
      double en = orc_rk_norm(pool, err, target, n_var);
      if (err_norms) err_norms[step] = en;
    }
    memcpy(x0, x_inout, (size_t)n_var * sizeof(double));
  }
  free(x0);
  free(ks);
  free(temp);
  free(err);
  free(target);
  orc_pool_destroy(pool);
  return 0;
}

/* One right-hand side evaluation dxdt = f(x) with n_threads (<= 1: serial). */
int orc_ode_rhs(const orc_ode* ode, const double* x, double* dxdt, int n_threads) {
  if (!ode || !x || !dxdt) return -1;
  orc_pool* pool = n_threads > 1 ? orc_pool_create(n_threads) : NULL;
  orc_ode_eval(pool, ode, x, dxdt);
  orc_pool_destroy(pool);
  return 0;
}

/* Timed repetitions of the RHS on one persistent pool (CPU baseline). */
int orc_ode_rhs_repeat(const orc_ode* ode, const double* x, double* dxdt, int n_threads,
                       int64_t reps) {
  if (!ode || !x || !dxdt) return -1;
  orc_pool* pool = n_threads > 1 ? orc_pool_create(n_threads) : NULL;
  for (int64_t r = 0; r < reps; ++r) orc_ode_eval(pool, ode, x, dxdt);
  orc_pool_destroy(pool);
  return 0;
}

/* Sampled-row accelerations in the i-owner form sum_{j != i, j ascending}
 * (x_j - x_i) / (|r|^2 + eps^2)^{3/2}, then * mass.  For serial pair order
 * this equals the reference sum bit for bit (body i receives its pair terms
 * in ascending partner order, and -(a/b) == (-a)/b).  Used to check rows of
 * very large systems whose full pair loop would take minutes. */
int orc_nbody_acc_rows(const orc_nbody* nb, const double* pos, const int64_t* rows,
                       int64_t n_rows, double* acc_rows) {
  if (!nb || !pos || !rows || !acc_rows) return -1;
  const int64_t n = nb->n_particles;
  const double eps2 = nb->softening * nb->softening;
  for (int64_t r = 0; r < n_rows; ++r) {
    int64_t i = rows[r];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t j = 0; j < n; ++j) {
      if (j == i) continue;
      double dx = pos[3 * j] - pos[3 * i];
      double dy = pos[3 * j + 1] - pos[3 * i + 1];
      double dz = pos[3 * j + 2] - pos[3 * i + 2];
      double dist_sq = dx * dx + dy * dy + dz * dz + eps2;
      double dist = sqrt(dist_sq);
      double den = dist * dist_sq;
      double ax = dx / den, ay = dy / den, az = dz / den;
      if (nb->masses) {
        ax *= nb->masses[j]; ay *= nb->masses[j]; az *= nb->masses[j];
      }
      sx += ax;
      sy += ay;
      sz += az;
    }
    if (!nb->masses && nb->mass != 0.0 && nb->mass != 1.0) {
      sx *= nb->mass;
      sy *= nb->mass;
      sz *= nb->mass;
    }
    acc_rows[3 * r] = sx;
    acc_rows[3 * r + 1] = sy;
    acc_rows[3 * r + 2] = sz;
  }
  return 0;
}

/* Energy and momentum diagnostics, restating scripts/nbody_physics/energy.py
 * (softened pair potential :146-173 and kinetic energy :191-192) with masses:
 * PE = -sum_{i<j} m_i m_j / sqrt(r^2 + eps^2), KE = sum m v^2 / 2.
 * out[0]=KE, out[1]=PE, out[2..4]=linear momentum, out[5..7]=angular momentum. */
int orc_nbody_energy(const orc_nbody* nb, const double* x, double* out) {
  if (!nb || !x || !out) return -1;
  const int64_t n = nb->n_particles;
  const double* pos = x;
  const double* vel = x + 3 * n;
  const double eps2 = nb->softening * nb->softening;
  double ke = 0.0, pe = 0.0, px = 0.0, py = 0.0, pz = 0.0, lx = 0.0, ly = 0.0, lz = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double mi = nb->masses ? nb->masses[i] : (nb->mass != 0.0 ? nb->mass : 1.0);
    double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    ke += mi * (vx * vx + vy * vy + vz * vz) / 2.0;
    px += mi * vx;
    py += mi * vy;
    pz += mi * vz;
    double rx = pos[3 * i], ry = pos[3 * i + 1], rz = pos[3 * i + 2];
    lx += mi * (ry * vz - rz * vy);
    ly += mi * (rz * vx - rx * vz);
    lz += mi * (rx * vy - ry * vx);
    double pei = 0.0;
    for (int64_t j = i + 1; j < n; ++j) {
      double mj = nb->masses ? nb->masses[j] : (nb->mass != 0.0 ? nb->mass : 1.0);
      double dx = pos[3 * j] - rx, dy = pos[3 * j + 1] - ry, dz = pos[3 * j + 2] - rz;
      pei -= mj / sqrt(dx * dx + dy * dy + dz * dz + eps2);
    }
    pe += mi * pei;
  }
  out[0] = ke;
  out[1] = pe;
  out[2] = px;
  out[3] = py;
  out[4] = pz;
  out[5] = lx;
  out[6] = ly;
  out[7] = lz;
  return 0;
}

/* Fixed-step leapfrog, LeapfrogParallel.hpp:11-41 with the kernels of :57-73
 * (pos += dt*(vel + 0.5*dt*acc); vel += 0.5*dt*(acc0 + acc1); acc0 = acc1),
 * accelerations from NBodyODE::acc (:41-46). */
int orc_leapfrog(const orc_nbody* nb, double* x_inout, double t0, double tf, double dt,
                 int64_t* n_steps_out) {
  if (!nb || !x_inout) return -1;
  const int64_t n_dof = 3 * nb->n_particles;
  double* pos = x_inout;
  double* vel = x_inout + n_dof;
  double* acc0 = (double*)calloc((size_t)n_dof, sizeof(double));
  double* acc1 = (double*)calloc((size_t)n_dof, sizeof(double));
  orc_pair_ctx pc = {nb, pos, acc0, nb->softening * nb->softening, 0};
  const int64_t n_pairs = nb->n_particles * (nb->n_particles - 1) / 2;
  orc_pair_task(&pc, 0, n_pairs, 0);
  if (!nb->masses && nb->mass != 0.0 && nb->mass != 1.0)
    for (int64_t i = 0; i < n_dof; ++i) acc0[i] *= nb->mass;
  double t = t0;
  int64_t steps = 0;
  while (t < tf) {
    for (int64_t i = 0; i < n_dof; ++i) pos[i] += dt * (vel[i] + 0.5 * dt * acc0[i]);
    memset(acc1, 0, (size_t)n_dof * sizeof(double));
    pc.acc = acc1;
    orc_pair_task(&pc, 0, n_pairs, 0);
    if (!nb->masses && nb->mass != 0.0 && nb->mass != 1.0)
      for (int64_t i = 0; i < n_dof; ++i) acc1[i] *= nb->mass;
    for (int64_t i = 0; i < n_dof; ++i) vel[i] += 0.5 * dt * (acc0[i] + acc1[i]);
    for (int64_t i = 0; i < n_dof; ++i) acc0[i] = acc1[i];
    t += dt;
    ++steps;
  }
  if (n_steps_out) *n_steps_out = steps;
  free(acc0);
  free(acc1);
  return 0;
}

/* std::mt19937 (Matsumoto & Nishimura 1998) and libstdc++'s
 * uniform_real_distribution<double>(a, b) via generate_canonical<double, 53>
 * (two 32-bit draws: (g1 + g2 * 2^32) / 2^64).  Reproduces the seeded cube of
 * src/test/SpinningCubeNBodyTest.hpp:37-57 and
 * src/demo/n_body_scenarios/SpinningParticlesInBox.hpp:41-66. */
typedef struct {
  uint32_t mt[624];
  int idx;
} orc_mt;

static void orc_mt_seed(orc_mt* g, uint32_t seed) {
  g->mt[0] = seed;
  for (int i = 1; i < 624; ++i)
    g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  g->idx = 624;
}

static uint32_t orc_mt_next(orc_mt* g) {
  if (g->idx >= 624) {
    for (int i = 0; i < 624; ++i) {
      uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
      g->mt[i] = g->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->idx = 0;
  }
  uint32_t y = g->mt[g->idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

static double orc_mt_canonical(orc_mt* g) {
  const double r = 4294967296.0;
  double sum = (double)orc_mt_next(g);
  sum += (double)orc_mt_next(g) * r;
  double ret = sum / (r * r);
  if (ret >= 1.0) ret = nextafter(1.0, 0.0);
  return ret;
}

/* Spinning uniform cube: n bodies, side L, positions U(0,L) per coordinate,
 * velocities (-omega*y, omega*x, 0) about the cube's vertical axis with
 * omega = 2*sqrt(pi/3)/sqrt(L^3/n). */
int orc_spinning_cube(int64_t n, double L, uint32_t seed, double* x_out) {
  if (!x_out || n < 1) return -1;
  orc_mt g;
  orc_mt_seed(&g, seed);
  const int64_t n_var = 6 * n;
  const double pi = 3.14159265358979323846;
  const double omega = 2.0 * sqrt(pi / 3.0) / sqrt(L * L * L / (double)n);
  for (int64_t i = 0; i < n_var / 2; ++i) x_out[i] = 0.0 + (L - 0.0) * orc_mt_canonical(&g);
  for (int64_t i = 0; i < n; ++i) {
    const double xx = x_out[3 * i] - L / 2.0;
    const double yy = x_out[3 * i + 1] - L / 2.0;
    x_out[n_var / 2 + 3 * i] = -omega * yy;
    x_out[n_var / 2 + 3 * i + 1] = omega * xx;
    x_out[n_var / 2 + 3 * i + 2] = 0.0;
  }
  return 0;
}

size_t orc_sizeof_tableau(void) { return sizeof(orc_tableau); }
size_t orc_sizeof_ode(void) { return sizeof(orc_ode); }
size_t orc_sizeof_stats(void) { return sizeof(orc_stats); }

/* ------------------------------------------------------------------------ */
/* Seeded Plummer sphere for the CPU-baseline legs of the benchmark, so      */
/* that they build their inputs without the GPU library: the same sampler   */
/* as the library's initial conditions (Aarseth, Henon & Wielen 1974:       */
/* r = a / sqrt(X^(-2/3) - 1) with X < 0.999, speed q sqrt(2) (1 + r^2 /    */
/* a^2)^(-1/4) / sqrt(a) with g(q) = q^2 (1 - q^2)^(7/2) by rejection,      */
/* isotropic directions, centre of mass removed), drawing from xoshiro256** */
/* seeded through splitmix64 (Blackman & Vigna), uniform doubles from the   */
/* top 53 bits.  The same seed gives the same bits as gb_ic_plummer.        */
/* ------------------------------------------------------------------------ */
typedef struct {
  uint64_t s[4];
} orc_rng;

static uint64_t orc_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static void orc_rng_seed(orc_rng* g, uint64_t seed) {
  uint64_t z = seed;
  for (int i = 0; i < 4; ++i) {
    z += 0x9e3779b97f4a7c15ULL;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    g->s[i] = x ^ (x >> 31);
  }
}

static uint64_t orc_rng_next(orc_rng* g) {
  uint64_t* s = g->s;
  const uint64_t r = orc_rotl(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = orc_rotl(s[3], 45);
  return r;
}

static double orc_uniform(orc_rng* g) {
  return (double)(orc_rng_next(g) >> 11) * (1.0 / 9007199254740992.0);
}

static void orc_unit_vector(orc_rng* g, double* x, double* y, double* z) {
  const double c = 2.0 * orc_uniform(g) - 1.0;
  const double ph = 6.283185307179586 * orc_uniform(g);
  const double s = sqrt(1.0 - c * c);
  *x = s * cos(ph);
  *y = s * sin(ph);
  *z = c;
}

int orc_ic_plummer(int64_t n, uint64_t seed, double a, double* x) {
  if (n < 2 || !x || !(a > 0.0)) return -1;
  orc_rng g;
  orc_rng_seed(&g, seed);
  for (int64_t i = 0; i < n; ++i) {
    double* p = x + 3 * i;
    double* v = x + 3 * n + 3 * i;
    double X;
    do X = orc_uniform(&g);
    while (X <= 0.0 || X >= 0.999);
    const double r = a / sqrt(pow(X, -2.0 / 3.0) - 1.0);
    double ux, uy, uz;
    orc_unit_vector(&g, &ux, &uy, &uz);
    p[0] = r * ux;
    p[1] = r * uy;
    p[2] = r * uz;
    double q, y;
    do {
      q = orc_uniform(&g);
      y = 0.1 * orc_uniform(&g);
    } while (y > q * q * pow(1.0 - q * q, 3.5));
    const double sp = q * sqrt(2.0) * pow(1.0 + r * r / (a * a), -0.25) / sqrt(a);
    orc_unit_vector(&g, &ux, &uy, &uz);
    v[0] = sp * ux;
    v[1] = sp * uy;
    v[2] = sp * uz;
  }
  double c[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      c[k] += x[3 * i + k];
      c[3 + k] += x[3 * n + 3 * i + k];
    }
  for (int k = 0; k < 6; ++k) c[k] /= (double)n;
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      x[3 * i + k] -= c[k];
      x[3 * n + 3 * i + k] -= c[3 + k];
    }
  return 0;
}
