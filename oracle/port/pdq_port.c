/*
 * pdq_port.c -- float64 C port of the reference algorithm for the isotropic
 * TS0 filter with adaptive steps (TEST INFRASTRUCTURE: CPU baseline and a
 * second check of the Python oracle; never part of the product).
 *
 * Follows the reference line by line, with dense generic linear algebra
 * (no structure exploitation), as XLA would run it on a CPU:
 *   system_matrices_1d_iwp / preconditioner_taylor  _probdiffeq/utilities.py:57-84
 *   IsotropicWienerIntegrated.transition            _probdiffeq/ssm_impl_isotropic.py:367-378
 *   IsotropicLatentCond.apply_flat/marginalise      ssm_impl_isotropic.py:75-89
 *   IsotropicLatentCond.revert                      ssm_impl_isotropic.py:107-133
 *   revert_conditional / sum_of_sqrtm_factors       util/cholesky_util.py:27-95
 *   IsotropicOdeTs0.linearize                       ssm_impl_isotropic.py:304-317
 *   solver / solver_mle / solver_dynamic            _probdiffeq/solvers.py:395-437, 549-599, 702-733
 *   error_residual_std                              solvers.py:925-996
 *   control_integral / control_proportional_integral _ivpsolve/controllers.py:24-84
 *   RejectionLoop, terminal values (clip_dt)        _ivpsolve/solvers_via_adaptive_steps.py:16-375
 *   jetexpand_ode_padded_scan                       _probdiffeq/jet_expansion_algorithms.py:49-103
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXN 8
#define MAXD 2
#define MAXR (2 * MAXN + 2)

/* ---------------- vector fields ---------------- */

static void vf_eval(int field, const double* p, const double* u, double* out) {
  switch (field) {
    case 0: { /* Lotka-Volterra */
      double y01 = u[0] * u[1];
      out[0] = p[0] * u[0] - p[1] * y01;
      out[1] = -p[2] * u[1] + p[3] * y01;
      break;
    }
    case 1: /* van der Pol */
      out[0] = u[1];
      out[1] = p[0] * ((1.0 - u[0] * u[0]) * u[1] - u[0]);
      break;
    default: /* FitzHugh-Nagumo */
      out[0] = p[2] * (u[0] - u[0] * u[0] * u[0] / 3.0 + u[1]);
      out[1] = -(1.0 / p[2]) * (u[0] - p[0] - p[1] * u[1]);
      break;
  }
}

/* Taylor series product of truncated series (normalised coefficients). */
static void ser_mul(const double* a, const double* b, double* r, int K) {
  for (int k = 0; k < K; ++k) {
    double s = 0;
    for (int j = 0; j <= k; ++j) s += a[j] * b[k - j];
    r[k] = s;
  }
}

/* Taylor-mode initial derivatives (num = nu) for the three 2-d fields. */
static void taylor_init(int field, const double* p, const double* y0, int nu, double tc[MAXN][MAXD]) {
  int K = nu + 1;
  double u0[MAXN] = {0}, u1[MAXN] = {0};
  u0[0] = y0[0];
  u1[0] = y0[1];
  for (int k = 0; k < nu; ++k) {
    double f0[MAXN] = {0}, f1[MAXN] = {0}, t[MAXN], t2[MAXN];
    if (field == 0) {
      ser_mul(u0, u1, t, K);
      for (int i = 0; i < K; ++i) {
        f0[i] = p[0] * u0[i] - p[1] * t[i];
        f1[i] = -p[2] * u1[i] + p[3] * t[i];
      }
    } else if (field == 1) {
      ser_mul(u0, u0, t, K);
      for (int i = 0; i < K; ++i) t2[i] = (i == 0 ? 1.0 : 0.0) - t[i];
      ser_mul(t2, u1, t, K);
      for (int i = 0; i < K; ++i) {
        f0[i] = u1[i];
        f1[i] = p[0] * (t[i] - u0[i]);
      }
    } else {
      ser_mul(u0, u0, t, K);
      ser_mul(t, u0, t2, K);
      for (int i = 0; i < K; ++i) {
        f0[i] = p[2] * (u0[i] - t2[i] / 3.0 + u1[i]);
        f1[i] = -(1.0 / p[2]) * (u0[i] - (i == 0 ? p[0] : 0.0) - p[1] * u1[i]);
      }
    }
    u0[k + 1] = f0[k] / (k + 1);
    u1[k + 1] = f1[k] / (k + 1);
  }
  double fact = 1.0;
  for (int k = 0; k < K; ++k) {
    if (k > 0) fact *= k;
    tc[k][0] = u0[k] * fact;
    tc[k][1] = u1[k] * fact;
  }
}

/* ---------------- dense linear algebra ---------------- */

/* R factor (cols x cols, upper) of a rows x cols matrix by Householder, like geqrf. */
static void qr_r(double M[MAXR][MAXR], int rows, int cols, double R[MAXR][MAXR]) {
  double A[MAXR][MAXR];
  memcpy(A, M, sizeof(A));
  for (int c = 0; c < cols && c < rows; ++c) {
    double nrm2 = 0;
    for (int r = c; r < rows; ++r) nrm2 += A[r][c] * A[r][c];
    if (nrm2 == 0) continue;
    double alpha = A[c][c], nrm = sqrt(nrm2);
    double beta = alpha >= 0 ? -nrm : nrm;
    double v[MAXR];
    v[c] = 1.0;
    for (int r = c + 1; r < rows; ++r) v[r] = A[r][c] / (alpha - beta);
    double tau = (beta - alpha) / beta;
    for (int j = c; j < cols; ++j) {
      double w = 0;
      for (int r = c; r < rows; ++r) w += v[r] * A[r][j];
      w *= tau;
      for (int r = c; r < rows; ++r) A[r][j] -= w * v[r];
    }
  }
  for (int i = 0; i < cols; ++i)
    for (int j = 0; j < cols; ++j) R[i][j] = (j >= i && i < rows) ? A[i][j] : 0.0;
}

typedef struct {
  double mean[MAXN][MAXD];
  double chol[MAXN][MAXN];
} Normal;

typedef struct {
  int field, nu, solver, control, d;
  double atol, rtol, eps, damp, safety, fmin, fmax, ei, ep;
  double A[MAXN][MAXN], Q[MAXN][MAXN];
} Setup;

static void precon(const Setup* s, double dt, double* p, double* pinv) {
  int n = s->nu + 1;
  for (int i = 0; i < n; ++i) {
    int pw = s->nu - i;
    double f = 1.0;
    for (int k = 2; k <= pw; ++k) f *= k;
    p[i] = pow(dt, pw) / f;
    pinv[i] = pow(dt, -pw) * f;
  }
}

/* transition(dt, scale).marginalise(rv) (ssm_impl_isotropic.py:81-89, 367-378) */
static void marginalise_prior(const Setup* s, const Normal* rv, double dt, double scale, Normal* out) {
  int n = s->nu + 1, d = s->d;
  double p[MAXN], pinv[MAXN];
  precon(s, dt, p, pinv);
  double sq = sqrt(fabs(dt)) * scale;
  double mean[MAXN][MAXD], chol[MAXN][MAXN];
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < d; ++j) mean[i][j] = pinv[i] * rv->mean[i][j];
    for (int j = 0; j < n; ++j) chol[i][j] = pinv[i] * rv->chol[i][j];
  }
  double M[MAXR][MAXR] = {{0}}, R[MAXR][MAXR];
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      double acc = 0;
      for (int k = 0; k < n; ++k) acc += s->A[c][k] * chol[k][r];
      M[r][c] = acc;                /* (A chol)^T */
      M[n + r][c] = sq * s->Q[c][r]; /* noise chol^T */
    }
  qr_r(M, 2 * n, n, R);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < d; ++j) {
      double acc = 0;
      for (int k = 0; k < n; ++k) acc += s->A[i][k] * mean[k][j];
      out->mean[i][j] = p[i] * acc;
    }
    for (int j = 0; j < n; ++j) out->chol[i][j] = fabs(p[i]) * R[j][i];
  }
}

typedef struct {
  double f[MAXD];  /* vector field at the linearisation point (bias mean = -f) */
} Ts0;

/* fx.revert(rv) with H = e_1, bias (-f, damp): corrected normal, observed chol (1x1), observed mean */
static void revert_ts0(const Setup* s, const Ts0* fx, const Normal* rv, Normal* cor, double* r_obs, double* mobs) {
  int n = s->nu + 1, d = s->d;
  double M[MAXR][MAXR] = {{0}}, R[MAXR][MAXR];
  M[0][0] = s->damp;
  for (int r = 0; r < n; ++r) {
    M[1 + r][0] = rv->chol[1][r];                           /* (H chol)^T */
    for (int c = 0; c < n; ++c) M[1 + r][1 + c] = rv->chol[c][r]; /* chol^T */
  }
  qr_r(M, n + 1, n + 1, R);
  double RY = R[0][0];
  double G[MAXN];
  for (int i = 0; i < n; ++i) G[i] = R[0][1 + i] / RY; /* solve_triu(R_Y, R12)^T */
  for (int j = 0; j < d; ++j) mobs[j] = rv->mean[1][j] - fx->f[j];
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < d; ++j) cor->mean[i][j] = rv->mean[i][j] - G[i] * mobs[j];
    for (int j = 0; j < n; ++j) cor->chol[i][j] = R[1 + j][1 + i];
  }
  *r_obs = RY;
}

typedef struct {
  const Setup* s;
  int64_t begin, end;
  const double *params, *y0;
  double t0, t1, dt0;
  double *mean_out, *chol_out, *scale_out;
  int *steps_out, *attempts_out;
} Job;

static void solve_one(const Setup* s, const double* p, const double* y0, double t0, double t1, double dt0, double* mean_out,
                      double* chol_out, double* scale_out, int* steps_out, int* attempts_out) {
  int n = s->nu + 1, d = s->d;
  double tc[MAXN][MAXD];
  taylor_init(s->field, p, y0, s->nu, tc);
  Normal x;
  memset(&x, 0, sizeof(x));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) x.mean[i][j] = tc[i][j];
  double t = t0, dt = dt0, pi_prev = 1.0, running = 0.0;
  double num_data = 0.0;
  int num_steps = 0, attempts = 0;
  while (t + s->eps < t1) {
    double ep = 0.9;
    Normal prop;
    double prop_running = running;
    while (ep < 1.0) {
      double h = fmin(dt, t1 - t); /* clip_dt */
      if (!(fabs(h) > 1e-14 * fmax(1.0, fabs(t))) || attempts > (1 << 24)) {
        *attempts_out = -1;
        return;
      }
      ++attempts;
      /* u = transition(dt, 1).apply_flat(mean) (for dynamic & error estimate) */
      double pp[MAXN], pinv[MAXN];
      precon(s, h, pp, pinv);
      double mp[MAXN][MAXD];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < d; ++j) {
          double acc = 0;
          for (int k = 0; k < n; ++k) acc += s->A[i][k] * pinv[k] * x.mean[k][j];
          mp[i][j] = pp[i] * acc;
        }
      /* noise chol of apply_flat: |p| sqrt|h| Q; fx.marginalise -> l */
      double sq = sqrt(fabs(h));
      double lrow2 = 0;
      for (int j = 0; j < n; ++j) {
        double v = fabs(pp[1]) * sq * s->Q[1][j];
        lrow2 += v * v;
      }
      double ell = sqrt(lrow2 + s->damp * s->damp);
      Ts0 fx;
      vf_eval(s->field, p, mp[0], fx.f);
      double mo2 = 0;
      for (int j = 0; j < d; ++j) {
        double r = mp[1][j] - fx.f[j];
        mo2 += (r / ell) * (r / ell);
      }
      double sigma_loc = sqrt(mo2) / sqrt((double)d);
      double scale = (s->solver == 2) ? sigma_loc : 1.0;
      Normal pred;
      marginalise_prior(s, &x, h, scale, &pred);
      double r_obs, mobs[MAXD];
      revert_ts0(s, &fx, &pred, &prop, &r_obs, mobs);
      if (s->solver == 1) {
        double nt = 0;
        for (int j = 0; j < d; ++j) nt += (mobs[j] / r_obs) * (mobs[j] / r_obs);
        nt = sqrt(nt) / sqrt((double)d);
        double x1 = sqrt(num_data / (num_data + 1)) * running;
        double x2 = sqrt(1.0 / (num_data + 1)) * nt;
        prop_running = hypot(x1, x2);
      }
      /* error_residual_std */
      double err = fabs(sigma_loc) * ell * h;
      double acc = 0;
      for (int j = 0; j < d; ++j) {
        double ref = fmax(fabs(x.mean[0][j]), fabs(prop.mean[0][j]));
        double rr = err / (s->atol + s->rtol * ref);
        acc += rr * rr;
      }
      double norm = sqrt(acc / d);
      ep = pow(norm, -1.0 / n);
      double factor;
      if (s->control == 0) {
        factor = s->safety * ep;
      } else {
        factor = s->safety * pow(ep, s->ei) * pow(ep / pi_prev, s->ep);
        if (ep >= 1.0) pi_prev = ep;
      }
      factor = fmax(s->fmin, fmin(factor, s->fmax));
      dt = factor * h;
      if (ep >= 1.0) {
        t = t + h;
        ++num_steps;
        x = prop;
        running = prop_running;
        if (s->solver == 1) num_data += 1.0;
      }
      if (isnan(ep)) {
        *attempts_out = -1;
        return;
      }
    }
  }
  double out_scale = 1.0;
  if (s->solver == 1) out_scale = running / sqrt((double)num_steps);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < d; ++j) mean_out[i * d + j] = x.mean[i][j];
    for (int j = 0; j < n; ++j) chol_out[i * n + j] = out_scale * x.chol[i][j];
  }
  *scale_out = out_scale;
  *steps_out = num_steps;
  *attempts_out = attempts;
}

static void* run_job(void* arg) {
  Job* j = (Job*)arg;
  const Setup* s = j->s;
  int n = s->nu + 1, d = s->d, P = s->field == 0 ? 4 : (s->field == 1 ? 1 : 3);
  for (int64_t b = j->begin; b < j->end; ++b)
    solve_one(s, j->params + b * P, j->y0 + b * d, j->t0, j->t1, j->dt0, j->mean_out + b * n * d,
              j->chol_out + b * n * n, j->scale_out + b, j->steps_out + b, j->attempts_out + b);
  return NULL;
}

/* Build A (flip Pascal) and Q (lower sqrt of flip Hilbert). */
static void system_matrices(Setup* s) {
  int nu = s->nu, n = nu + 1;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (j < i) {
        s->A[i][j] = 0;
      } else {
        int N = nu - i, k = nu - j;
        double c = 1;
        for (int q = 1; q <= k; ++q) c = c * (N - k + q) / q;
        s->A[i][j] = c;
      }
    }
  long double C[MAXN][MAXN] = {{0}};
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      long double v = 1.0L / (2 * nu + 1 - i - j);
      for (int k = 0; k < j; ++k) v -= C[i][k] * C[j][k];
      C[i][j] = (i == j) ? sqrtl(v) : v / C[j][j];
    }
  for (int i = 0; i < MAXN; ++i)
    for (int j = 0; j < MAXN; ++j) s->Q[i][j] = (i < n && j <= i) ? (double)C[i][j] : 0.0;
}

/* Terminal-value solves of B instances on `threads` threads; returns 0. */
int pdq_port_solve_iso(int field, int nu, int solver, int control, double atol, double rtol, double t0, double t1,
                       double dt0, int64_t B, const double* params, const double* y0, int threads, double* mean_out,
                       double* chol_out, double* scale_out, int* steps_out, int* attempts_out) {
  if (nu < 1 || nu + 1 > MAXN || threads < 1) return 1;
  Setup s;
  memset(&s, 0, sizeof(s));
  s.field = field;
  s.nu = nu;
  s.solver = solver;
  s.control = control;
  s.d = 2;
  s.atol = atol;
  s.rtol = rtol;
  s.eps = 1e-8;
  s.damp = 0.0;
  s.safety = 0.95;
  s.fmin = 0.2;
  s.fmax = 10.0;
  s.ei = 0.3;
  s.ep = 0.4;
  system_matrices(&s);
  if (threads > B) threads = (int)(B > 0 ? B : 1);
  pthread_t tid[256];
  Job jobs[256];
  if (threads > 256) threads = 256;
  for (int i = 0; i < threads; ++i) {
    jobs[i] = (Job){&s, B * i / threads, B * (i + 1) / threads, params, y0, t0, t1, dt0, mean_out, chol_out, scale_out,
                    steps_out, attempts_out};
    pthread_create(&tid[i], NULL, run_job, &jobs[i]);
  }
  for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
  return 0;
}
