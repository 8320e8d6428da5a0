/*
 * fvoracle.c -- CPU restatement of the reference's residual evaluation and
 * RK stage update on the flattened mesh tables (include/fvgpu.h layout).
 *
 * TEST INFRASTRUCTURE ONLY.  Loaded by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arms as the checker; the product path
 * (libfvgpu) never calls it.
 *
 * Every function states the reference file:line it follows.  Expressions are
 * written in the reference's order of operations (C evaluates a+b+c as
 * (a+b)+c), so that, compiled with -ffp-contract=off, the results are
 * bit-identical to the reference's own C code compiled the same way; this is
 * checked against oracle/_ref (the reference sources compiled unchanged) by
 * tests/test_oracle_ref.py.  pow(x, 2.0) appears as x*x: GCC folds it to that
 * product at -O1 and above, so the compiled reference multiplies too.
 *
 * Layouts: U, UN, R [neq][n]; SF [6][neq][n]; SG [neq+1][3][n].
 *
 * Pieces with no reference code (the reference leaves them undefined or
 * absent) are restated from the mathematics and marked so: reflective and
 * no-slip ghost states (bc.c:38,42 call undefined functions), the CFL time
 * step (dt is a fixed input in the reference, inputset.c:90).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fvgpu.h"

#define NEQMAX 5

static const int kOpp[6] = {2, 3, 0, 1, 5, 4}; /* fcopp, operatetp.c:481-490 */

/* error reporting mirrors the device error word of libfvgpu */
#define FVO_ERR_NONFINITE 1
#define FVO_ERR_EOS 2
#define FVO_ERR_REGION 3
static int64_t g_err_cell = -1;
static int g_err_code = 0;
static void set_err(int code, int64_t cell) {
#pragma omp critical(fvo_err)
  {
    if (g_err_code == 0) {
      g_err_code = code;
      g_err_cell = cell;
    }
  }
}

/* Cells are independent in every per-cell loop below, so running them on
 * several threads gives the same bits as one thread. */
#ifdef _OPENMP
#include <omp.h>
void fvo_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}
int fvo_get_threads(void) { return omp_get_max_threads(); }
#else
void fvo_set_threads(int n) { (void)n; }
int fvo_get_threads(void) { return 1; }
#endif
int fvo_error(int64_t *cell) {
  if (cell) *cell = g_err_cell;
  return g_err_code;
}
void fvo_clear_error(void) {
  g_err_code = 0;
  g_err_cell = -1;
}

static int neq_of(const fvgpu_config *cfg) { return cfg->model == 2 ? 4 : 5; }

/* face state: the SOL fields the residual reads (strdata.h:360-402) */
typedef struct fstate {
  double r, u, v, w, e, p, c, ymass;
  double vec[NEQMAX];
  double ux, uy, uz, vx, vy, vz, wx, wy, wz;
} fstate;

/* ---- equations of state --------------------------------------------------- */

/* barotropic_eos, barotropic_eos.c:3-30 */
static void eos_barotropic(fstate *s) {
  const double nexp = 7.15, beta = 293526643.0, cbar = 1450.0, psat = 2339.0, rsat = 998.2;
  if (s->r >= rsat) {
    s->p = psat + beta * (pow((s->r / rsat), nexp) - 1.0);
    s->c = sqrt(beta * nexp * (pow((s->r / rsat), (nexp - 1))) / rsat);
  }
  if (s->r < rsat) {
    s->p = psat + cbar * ((1.0 / rsat) - (1.0 / s->r));
    s->c = sqrt(cbar / ((s->r) * (s->r)));
  }
}

/* barotropic_multiphase_eos, barotropic_eos.c:32-129 */
static int eos_mixture(fstate *s) {
  const double R_G = 286.0, T_ref = 293.15, r_sat = 998.1618, p_sat = 2340.0;
  const double c_liq = 1482.5, c_mixture = 1.0;
  double c_temp = c_liq;
  double b_coef = c_temp * c_temp * r_sat - p_sat - s->r * s->ymass * R_G * T_ref -
                  s->r * (c_temp * c_temp) * (1.0 - s->ymass);
  double d_coef = (p_sat - c_temp * c_temp * r_sat) * s->r * s->ymass * R_G * T_ref;
  double check = sqrt(b_coef * b_coef - 4.0 * d_coef);
  if (isnan(check)) {
    c_temp = c_mixture;
    b_coef = c_temp * c_temp * r_sat - p_sat - s->r * s->ymass * R_G * T_ref -
             s->r * (c_temp * c_temp) * (1.0 - s->ymass);
    d_coef = (p_sat - c_temp * c_temp * r_sat) * s->r * s->ymass * R_G * T_ref;
    check = sqrt(b_coef * b_coef - 4.0 * d_coef);
    if (isnan(check)) {
      s->p = NAN;
      s->c = c_temp;
      return FVO_ERR_EOS; /* the reference prints " double nan " and exits */
    }
  }
  const double p1 = (-b_coef + sqrt(b_coef * b_coef - 4.0 * d_coef)) / 2.0;
  const double p2 = (-b_coef - sqrt(b_coef * b_coef - 4.0 * d_coef)) / 2.0;
  s->p = ((p1) > (p2)) ? (p1) : (p2);
  s->c = c_temp;
  return 0;
}

/* Face state from conservative values q (facercnstr.c:20-59 when `clip`,
 * facevalues.c:113-142 otherwise).  grad: SG of the cell the values come
 * from, or NULL when ns == 0 (facercnstr.c:73-85). */
static int face_state(const fvgpu_config *cfg, const double *q, int clip, const double *grad9,
                      fstate *s) {
  int rc = 0;
  s->r = q[0];
  s->u = q[1] / s->r;
  s->v = q[2] / s->r;
  s->w = q[3] / s->r;
  s->vec[0] = s->r;
  s->vec[1] = q[1];
  s->vec[2] = q[2];
  s->vec[3] = q[3];
  if (cfg->model == 1) {
    s->e = q[4];
    s->vec[4] = q[4];
    const double e_int = (s->e / s->r) - 0.5 * (s->u * s->u + s->v * s->v + s->w * s->w);
    s->p = s->r * (cfg->gamma - 1.0) * e_int - cfg->gamma * cfg->pinf;
    s->c = sqrt(cfg->gamma * (s->p + cfg->pinf) / s->r);
  } else if (cfg->model == 2) {
    eos_barotropic(s);
  } else if (cfg->model == 3) {
    s->ymass = q[4] / s->r;
    s->vec[4] = q[4];
    if (clip) {
      if (s->ymass < (cfg->ymin / 1000.0)) s->ymass = (cfg->ymin / 1000.0);
      if (s->ymass > (1.0 - (cfg->ymin / 1000.0))) s->ymass = 1.0 - (cfg->ymin / 1000.0);
    }
    rc = eos_mixture(s);
  }
  if (grad9) {
    s->ux = grad9[0];
    s->uy = grad9[1];
    s->uz = grad9[2];
    s->vx = grad9[3];
    s->vy = grad9[4];
    s->vz = grad9[5];
    s->wx = grad9[6];
    s->wy = grad9[7];
    s->wz = grad9[8];
  }
  return rc;
}

/* Ghost state of a boundary face: bc(), bc.c:19-49.  The ghost starts as a
 * copy of the own state (residual_faces_AMR.c:196-198, 207-209). */
static void apply_bc(const fvgpu_config *cfg, int bc, const double *frame, fstate *g) {
  if (bc == 1) {
    /* bc_inlet.c -> asinvalues.c:7-44 on the configured inflow state
     * (model 1; the model-3 variant writes its EOS into the other side,
     * asinvalues_multiphase.c:22, and is not supported) */
    const double *q = cfg->inflow;
    const double rho = q[0];
    g->r = rho;
    g->u = q[1] / rho;
    g->v = q[2] / rho;
    g->w = q[3] / rho;
    g->vec[0] = rho;
    g->vec[1] = q[1];
    g->vec[2] = q[2];
    g->vec[3] = q[3];
    g->e = q[4];
    g->vec[4] = q[4];
    const double e_int = (q[4] / rho) - 0.5 * (g->u * g->u + g->v * g->v + g->w * g->w);
    g->p = g->r * (cfg->gamma - 1.0) * e_int - cfg->gamma * cfg->pinf;
    g->c = sqrt(cfg->gamma * (g->p + cfg->pinf) / g->r);
  } else if (bc == 3 || bc == 4) {
    /* Restated from the mathematics (no reference code): slip wall mirrors
     * the normal velocity, no-slip wall reverses the velocity; density,
     * pressure and sound speed are kept. */
    double un = 0.0;
    if (bc == 3) un = (g->u * frame[0] + g->v * frame[1]) + g->w * frame[2];
    if (bc == 3) {
      g->u = g->u - 2.0 * un * frame[0];
      g->v = g->v - 2.0 * un * frame[1];
      g->w = g->w - 2.0 * un * frame[2];
      /* the momentum mirrored as such: exact on axis-aligned faces */
      const double mn = (g->vec[1] * frame[0] + g->vec[2] * frame[1]) + g->vec[3] * frame[2];
      g->vec[1] = g->vec[1] - 2.0 * mn * frame[0];
      g->vec[2] = g->vec[2] - 2.0 * mn * frame[1];
      g->vec[3] = g->vec[3] - 2.0 * mn * frame[2];
    } else {
      g->u = -g->u;
      g->v = -g->v;
      g->w = -g->w;
      g->vec[1] = -g->vec[1];
      g->vec[2] = -g->vec[2];
      g->vec[3] = -g->vec[3];
    }
  }
  /* bc == 2 (outflow): the ghost is the own state, bc.c:26-30 */
}

/* ---- HLLC --------------------------------------------------------------------- */

/* flux_adv, flux_adv.c:10-45; st = p I (facercnstr.c:61-71) */
static void flux_adv(const fvgpu_config *cfg, const fstate *s, double F[NEQMAX][3]) {
  F[0][0] = s->u * s->r;
  F[0][1] = s->v * s->r;
  F[0][2] = s->w * s->r;
  F[1][0] = s->r * s->u * s->u + s->p;
  F[1][1] = s->r * s->u * s->v + 0.0;
  F[1][2] = s->r * s->u * s->w + 0.0;
  F[2][0] = s->r * s->v * s->u + 0.0;
  F[2][1] = s->r * s->v * s->v + s->p;
  F[2][2] = s->r * s->v * s->w + 0.0;
  F[3][0] = s->r * s->w * s->u + 0.0;
  F[3][1] = s->r * s->w * s->v + 0.0;
  F[3][2] = s->r * s->w * s->w + s->p;
  if (cfg->model == 1) {
    F[4][0] = s->u * (s->e + s->p);
    F[4][1] = s->v * (s->e + s->p);
    F[4][2] = s->w * (s->e + s->p);
  }
  if (cfg->model == 3) {
    F[4][0] = s->u * s->r * s->ymass;
    F[4][1] = s->v * s->r * s->ymass;
    F[4][2] = s->w * s->r * s->ymass;
  }
}

/* (R st R^T)[0][0] for st = p I, rotate_vectors.c:32-90 */
static double rotate_s11(const double *fr, double p) {
  const double vec[3][3] = {{fr[0], fr[1], fr[2]}, {fr[3], fr[4], fr[5]}, {fr[6], fr[7], fr[8]}};
  const double st[3][3] = {{p, 0.0, 0.0}, {0.0, p, 0.0}, {0.0, 0.0, p}};
  double m1[3] = {0.0, 0.0, 0.0};
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) m1[j] += vec[0][k] * st[k][j];
  double m2 = 0.0;
  for (int k = 0; k < 3; ++k) m2 += m1[k] * vec[0][k];
  return m2;
}

/* star_region_euler, star_region_euler.c:3-40 */
static void star_state(const fvgpu_config *cfg, const fstate *s, const double *fr, double S_S,
                       double SK, double uK, double vK, double wK, double Us[NEQMAX]) {
  const double const_S = s->r * (SK - uK) / (SK - S_S);
  const double u = S_S, v = vK, w = wK;
  Us[0] = const_S;
  Us[1] = const_S * (u * fr[0] + v * fr[3] + w * fr[6]);
  Us[2] = const_S * (u * fr[1] + v * fr[4] + w * fr[7]);
  Us[3] = const_S * (u * fr[2] + v * fr[5] + w * fr[8]);
  if (cfg->model == 1)
    Us[4] = const_S * ((s->e / s->r) + (S_S - uK) * (S_S + (s->p / (s->r * (SK - uK)))));
  if (cfg->model == 3) Us[4] = const_S * s->ymass;
}

/* hllc_euler + compute_wave_speeds: hllc_euler.c:3-55,
 * compute_wave_speeds.c:3-88.  Returns 0 or FVO_ERR_REGION. */
static int hllc(const fvgpu_config *cfg, const fstate *L, const fstate *R, const double *fr,
                int bc, double F[NEQMAX][3], double FH[NEQMAX]) {
  const int neq = neq_of(cfg);
  const double nx = fr[0], ny = fr[1], nz = fr[2];
  const double mx = fr[3], my = fr[4], mz = fr[5];
  const double lx = fr[6], ly = fr[7], lz = fr[8];
  const double uL = L->u * nx + L->v * ny + L->w * nz;
  const double vL = L->u * mx + L->v * my + L->w * mz;
  const double wL = L->u * lx + L->v * ly + L->w * lz;
  const double uR = R->u * nx + R->v * ny + R->w * nz;
  const double vR = R->u * mx + R->v * my + R->w * mz;
  const double wR = R->u * lx + R->v * ly + R->w * lz;
  const double ruL = L->r * uL;
  const double ruR = R->r * uR;
  const double cL = L->c, cR = R->c;
  const double SR = (((uL + cL)) > ((uR + cR))) ? ((uL + cL)) : ((uR + cR));
  const double SL = (((uL - cL)) < ((uR - cR))) ? ((uL - cL)) : ((uR - cR));
  const double s11L = rotate_s11(fr, L->p);
  const double s11R = rotate_s11(fr, R->p);
  double S_S = ((L->r * (uL * uL) + s11L) - (R->r * (uR * uR) + s11R) - (SL * ruL) + (SR * ruR)) /
               (ruL - ruR - (SL * L->r) + (SR * R->r));
  /* compute_wave_speeds.c:173-176 stops the run on a NaN S* */
  const int bad_speed = isnan(S_S);
  for (int iv = 0; iv < neq; ++iv) FH[iv] = 0.0;
  if (bc == 3) S_S = 0.0;
  double Us[NEQMAX];
  if (0.0 <= SL) {
    flux_adv(cfg, L, F);
  } else if ((SL <= 0.0) && (0.0 <= S_S)) {
    star_state(cfg, L, fr, S_S, SL, uL, vL, wL, Us);
    flux_adv(cfg, L, F);
    for (int iv = 0; iv < neq; ++iv) FH[iv] = SL * (Us[iv] - L->vec[iv]);
  } else if ((S_S <= 0.0) && (0.0 <= SR)) {
    star_state(cfg, R, fr, S_S, SR, uR, vR, wR, Us);
    flux_adv(cfg, R, F);
    for (int iv = 0; iv < neq; ++iv) FH[iv] = SR * (Us[iv] - R->vec[iv]);
  } else if (SR <= 0.0) {
    flux_adv(cfg, R, F);
  } else {
    for (int iv = 0; iv < neq; ++iv) {
      FH[iv] = NAN;
      F[iv][0] = F[iv][1] = F[iv][2] = NAN;
    }
    return FVO_ERR_REGION; /* "stop if", hllc_euler.c:52-55 */
  }
  return bad_speed ? FVO_ERR_REGION : 0;
}

/* flux_viscous, flux_viscous.c:57-232 with turb = 0 (mu_turb = 0) */
static void flux_visc(const fvgpu_config *cfg, const fstate *s, const fstate *s1,
                      double FV[NEQMAX][3]) {
  const double uf = 0.5 * (s->u + s1->u);
  const double vf = 0.5 * (s->v + s1->v);
  const double wf = 0.5 * (s->w + s1->w);
  const double ux = 0.5 * (s->ux + s1->ux), uy = 0.5 * (s->uy + s1->uy), uz = 0.5 * (s->uz + s1->uz);
  const double vx = 0.5 * (s->vx + s1->vx), vy = 0.5 * (s->vy + s1->vy), vz = 0.5 * (s->vz + s1->vz);
  const double wx = 0.5 * (s->wx + s1->wx), wy = 0.5 * (s->wy + s1->wy), wz = 0.5 * (s->wz + s1->wz);
  const double mu = cfg->visc + 0.0;
  const double txx = mu * (2.0 * ux - (2.0 / 3.0) * (ux + vy + wz));
  const double tyy = mu * (2.0 * vy - (2.0 / 3.0) * (ux + vy + wz));
  const double tzz = mu * (2.0 * wz - (2.0 / 3.0) * (ux + vy + wz));
  const double txy = mu * (uy + vx);
  const double txz = mu * (uz + wx);
  const double tyz = mu * (vz + wy);
  const double tyx = txy, tzy = tyz, tzx = txz;
  FV[0][0] = 0.0;
  FV[0][1] = 0.0;
  FV[0][2] = 0.0;
  FV[1][0] = txx;
  FV[1][1] = tyx;
  FV[1][2] = tzx;
  FV[2][0] = txy;
  FV[2][1] = tyy;
  FV[2][2] = tzy;
  FV[3][0] = txz;
  FV[3][1] = tyz;
  FV[3][2] = tzz;
  if (cfg->eos == 1) {
    FV[4][0] = uf * txx + vf * txy + wf * txz;
    FV[4][1] = uf * tyx + vf * tyy + wf * tyz;
    FV[4][2] = uf * tzx + vf * tzy + wf * tzz;
  }
}

/* ---- helpers on the tables ----------------------------------------------------- */

static void load_cell(const double *U, int neq, int64_t n, int64_t c, double *q) {
  for (int v = 0; v < neq; ++v) q[v] = U[(int64_t)v * n + c];
}

/* ---- faceinterp ------------------------------------------------------------------
 * faceinterp.c:21-61 with distance (precomputed in the tables, distance.c),
 * deltavalues.c:3-26, facevalues_MUSCL.c:3-56, reconctruct_V3.c:3-57
 * (iprimtv = 0). */

/* deltavalues(run, crnt, delta, f): neighbour (or ghost) minus own */
static void delta_values(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U,
                         int64_t c, int f, const double *own, double *delta) {
  const int neq = neq_of(cfg);
  const int64_t n = m->ncells;
  const int32_t code = m->nbr[(int64_t)f * n + c];
  double nb[NEQMAX];
  if (code >= 0) {
    load_cell(U, neq, n, code, nb);
  } else if (code <= FVGPU_HANG0) {
    const int32_t *k = m->hang_nbr + 4 * (int64_t)(FVGPU_HANG0 - code);
    for (int v = 0; v < neq; ++v) nb[v] = 0.0;
    for (int s = 0; s < 4; ++s)
      for (int v = 0; v < neq; ++v) nb[v] += U[(int64_t)v * n + k[s]] / ((double)4);
  } else {
    /* boundary: own values, then bc() on the ghost (deltavalues.c:9-14) */
    fstate g;
    memset(&g, 0, sizeof g);
    for (int v = 0; v < neq; ++v) g.vec[v] = own[v];
    const int bc = -1 - code;
    if (bc == 1 || bc == 3 || bc == 4) {
      /* ghost needs the primitive fields bc() reads */
      face_state(cfg, own, 0, NULL, &g);
      apply_bc(cfg, bc, m->frames + 9 * f, &g);
    }
    for (int v = 0; v < neq; ++v) nb[v] = g.vec[v];
  }
  for (int v = 0; v < neq; ++v) delta[v] = nb[v] - own[v];
}

void fvo_faceinterp(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, double *SF) {
  const int neq = neq_of(cfg);
  const int64_t n = m->ncells;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < n; ++c) {
    double own[NEQMAX];
    load_cell(U, neq, n, c, own);
    for (int f = 0; f < 6; ++f) {
      const int fo = kOpp[f];
      const double dist_p1_cf = m->dcf[(int64_t)f * n + c];
      const double dist_p1_cc = m->dcc[(int64_t)f * n + c];
      const double dist_m1_cc = m->dcc[(int64_t)fo * n + c];
      double delta0[NEQMAX], delta1[NEQMAX];
      delta_values(cfg, m, U, c, fo, own, delta1);
      delta_values(cfg, m, U, c, f, own, delta0);
      const int bcf = m->nbr[(int64_t)f * n + c] < 0 && m->nbr[(int64_t)f * n + c] > FVGPU_HANG0;
      for (int iv = 0; iv < neq; ++iv) {
        double grad = 0.0;
        if (!bcf) {
          if (fabs(delta0[iv]) > 1e-10) { /* pow(10.0,-10.0) == 1e-10 */
            const double product = (-delta1[iv] / dist_m1_cc) * (delta0[iv] / dist_p1_cc);
            if (product > 0.0) {
              if (fabs(-delta1[iv] / dist_m1_cc) > fabs(delta0[iv] / dist_p1_cc))
                grad = delta0[iv] / dist_p1_cc;
              else
                grad = -delta1[iv] / dist_m1_cc;
            } else {
              grad = 0.0;
            }
          }
        }
        SF[((int64_t)f * neq + iv) * n + c] = own[iv] + dist_p1_cf * grad;
      }
    }
  }
}

/* ---- gradcalc ----------------------------------------------------------------------
 * gradcalc.c:9-47: Green-Gauss over sub-faces with first-order face values
 * (facevalues.c) and the EOS pressure as variable neq. */
void fvo_gradcalc(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, double *SG) {
  const int neq = neq_of(cfg);
  const int64_t n = m->ncells;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < n; ++c) {
    double g[NEQMAX + 1][3];
    for (int iv = 0; iv <= neq; ++iv) g[iv][0] = g[iv][1] = g[iv][2] = 0.0;
    double own[NEQMAX];
    load_cell(U, neq, n, c, own);
    const double Vol = m->vol[c];
    for (int f = 0; f < 6; ++f) {
      const int32_t code = m->nbr[(int64_t)f * n + c];
      const double *fr = m->frames + 9 * f;
      const int nsub = code <= FVGPU_HANG0 ? 4 : 1;
      for (int ing = 0; ing < nsub; ++ing) {
        fstate s, s1;
        memset(&s, 0, sizeof s);
        memset(&s1, 0, sizeof s1);
        if (face_state(cfg, own, 0, NULL, &s)) set_err(FVO_ERR_EOS, c);
        double A;
        if (code >= 0) {
          double q[NEQMAX];
          load_cell(U, neq, n, code, q);
          if (face_state(cfg, q, 0, NULL, &s1)) set_err(FVO_ERR_EOS, c);
          A = m->area[(int64_t)f * n + c];
        } else if (code <= FVGPU_HANG0) {
          const int64_t r = FVGPU_HANG0 - code;
          double q[NEQMAX];
          load_cell(U, neq, n, m->hang_nbr[4 * r + ing], q);
          if (face_state(cfg, q, 0, NULL, &s1)) set_err(FVO_ERR_EOS, c);
          A = m->hang_area[4 * r + ing];
        } else {
          face_state(cfg, own, 0, NULL, &s1);
          apply_bc(cfg, -1 - code, fr, &s1);
          A = m->area[(int64_t)f * n + c];
        }
        for (int iv = 0; iv < neq; ++iv) {
          g[iv][0] += 0.5 * (s1.vec[iv] + s.vec[iv]) * fr[0] * A / Vol;
          g[iv][1] += 0.5 * (s1.vec[iv] + s.vec[iv]) * fr[1] * A / Vol;
          g[iv][2] += 0.5 * (s1.vec[iv] + s.vec[iv]) * fr[2] * A / Vol;
        }
        g[neq][0] += 0.5 * (s1.p + s.p) * fr[0] * A / Vol;
        g[neq][1] += 0.5 * (s1.p + s.p) * fr[1] * A / Vol;
        g[neq][2] += 0.5 * (s1.p + s.p) * fr[2] * A / Vol;
      }
    }
    for (int iv = 0; iv <= neq; ++iv)
      for (int d = 0; d < 3; ++d) SG[((int64_t)iv * 3 + d) * n + c] = g[iv][d];
  }
}

/* ---- residual ----------------------------------------------------------------------
 * RHS.c:3-13 -> residual_faces_AMR.c:10-202 (every face evaluated from both
 * sides, sub-faces of a 1:4 face in table order).  `inner` selects the
 * RHS_nb variant (RHS_nb.c:3-15): only cells with inner[c] == inner_outer are
 * evaluated; inner == NULL evaluates all. */
static void grad9_of(const double *SG, int64_t n, int64_t c, double *g9) {
  /* SG[1..3][0..2]: gradients of rho u, rho v, rho w (facercnstr.c:73-85) */
  for (int a = 0; a < 3; ++a)
    for (int d = 0; d < 3; ++d) g9[a * 3 + d] = SG[((int64_t)(1 + a) * 3 + d) * n + c];
}

void fvo_rhs_nb(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U,
                const double *SF, const double *SG, double *R, const int32_t *inner,
                int inner_outer) {
  const int neq = neq_of(cfg);
  const int64_t n = m->ncells;
  const int muscl = cfg->ischeme == 2;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < n; ++c) {
    if (inner && inner[c] != inner_outer) continue;
    double rhs[NEQMAX];
    double FV[NEQMAX][3];
    for (int iv = 0; iv < neq; ++iv) {
      rhs[iv] = 0.0;
      FV[iv][0] = FV[iv][1] = FV[iv][2] = 0.0;
    }
    double g9own[9];
    if (cfg->ns == 1) grad9_of(SG, n, c, g9own);
    for (int f = 0; f < 6; ++f) {
      const int32_t code = m->nbr[(int64_t)f * n + c];
      const double *fr = m->frames + 9 * f;
      const int boundary = code < 0 && code > FVGPU_HANG0;
      const int Nneig = code <= FVGPU_HANG0 ? 4 : 1;
      double flux_face[NEQMAX];
      for (int iv = 0; iv < neq; ++iv) flux_face[iv] = 0.0;
      double qown[NEQMAX];
      for (int v = 0; v < neq; ++v)
        qown[v] = muscl ? SF[((int64_t)f * neq + v) * n + c] : U[(int64_t)v * n + c];
      fstate s;
      memset(&s, 0, sizeof s);
      if (face_state(cfg, qown, muscl, cfg->ns == 1 ? g9own : NULL, &s)) set_err(FVO_ERR_EOS, c);
      for (int ineig = 0; ineig < Nneig; ++ineig) {
        fstate s1;
        memset(&s1, 0, sizeof s1);
        double A;
        if (boundary) {
          if (face_state(cfg, qown, muscl, cfg->ns == 1 ? g9own : NULL, &s1)) set_err(FVO_ERR_EOS, c);
          apply_bc(cfg, -1 - code, fr, &s1);
          A = m->area[(int64_t)f * n + c];
        } else {
          int64_t k;
          if (code >= 0) {
            k = code;
            A = m->area[(int64_t)f * n + c];
          } else {
            const int64_t r = FVGPU_HANG0 - code;
            k = m->hang_nbr[4 * r + ineig];
            A = m->hang_area[4 * r + ineig];
          }
          const int nf = m->nbr_face[(int64_t)f * n + c];
          double q[NEQMAX], g9[9];
          for (int v = 0; v < neq; ++v)
            q[v] = muscl ? SF[((int64_t)nf * neq + v) * n + k] : U[(int64_t)v * n + k];
          if (cfg->ns == 1) grad9_of(SG, n, k, g9);
          if (face_state(cfg, q, muscl, cfg->ns == 1 ? g9 : NULL, &s1)) set_err(FVO_ERR_EOS, c);
        }
        if (cfg->ns == 1) flux_visc(cfg, &s, &s1, FV);
        double F[NEQMAX][3], FH[NEQMAX];
        if (hllc(cfg, &s, &s1, fr, boundary ? -1 - code : 0, F, FH)) set_err(FVO_ERR_REGION, c);
        for (int iv = 0; iv < neq; ++iv)
          flux_face[iv] += -(A) * (((F[iv][0] - FV[iv][0]) * fr[0] + (F[iv][1] - FV[iv][1]) * fr[1] +
                                    (F[iv][2] - FV[iv][2]) * fr[2]) +
                                   FH[iv]);
      }
      for (int iv = 0; iv < neq; ++iv) rhs[iv] += flux_face[iv];
    }
    for (int iv = 0; iv < neq; ++iv) {
      if (isnan(rhs[iv])) set_err(FVO_ERR_NONFINITE, c);
      R[(int64_t)iv * n + c] = rhs[iv];
    }
  }
}

void fvo_rhs(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, const double *SF,
             const double *SG, double *R) {
  fvo_rhs_nb(cfg, m, U, SF, SG, R, NULL, 0);
}

/* ---- RK stage update, RK.c:3-56 --------------------------------------------------- */
void fvo_rk(int irk, double dt, int neq, const fvgpu_mesh_soa *m, double *S, double *SN,
            const double *RHS) {
  const int64_t n = m->ncells;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < n; ++c) {
    const double Vol = m->vol[c];
    for (int e = 0; e < neq; ++e) {
      const int64_t i = (int64_t)e * n + c;
      switch (irk) {
        case 0:
          SN[i] = S[i];
          break;
        case 1:
          S[i] = SN[i] + dt * (1.0 / Vol) * RHS[i];
          break;
        case 2:
          S[i] = (3.0 / 4.0) * SN[i] + (1.0 / 4.0) * S[i] + (1.0 / 4.0) * dt * RHS[i] / Vol;
          break;
        case 3:
          S[i] = (1.0 / 3.0) * SN[i] + (2.0 / 3.0) * S[i] + (2.0 / 3.0) * dt * RHS[i] / Vol;
          break;
        case 4:
          S[i] = (1.0 / 2.0) * SN[i] + (1.0 / 2.0) * S[i] + (1.0 / 2.0) * dt * RHS[i] / Vol;
          break;
        default:
          break;
      }
    }
  }
}

/* One time step: RK(0), then per stage faceinterp -> gradcalc -> RHS -> RK(k)
 * (the stage body of the missing advancetimeexplicit, loop.c:48).  Scratch
 * SF, SG, R is caller-allocated. */
void fvo_step(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const int *stages, int nstages,
              double dt, double *S, double *SN, double *SF, double *SG, double *R) {
  const int neq = neq_of(cfg);
  fvo_rk(0, dt, neq, m, S, SN, R);
  for (int k = 0; k < nstages; ++k) {
    if (cfg->ischeme == 2) fvo_faceinterp(cfg, m, S, SF);
    if (cfg->ns == 1) fvo_gradcalc(cfg, m, S, SG);
    fvo_rhs(cfg, m, S, SF, SG, R);
    fvo_rk(stages[k], dt, neq, m, S, SN, R);
  }
}

/* ---- conservation sums, conservationcalc.c:19-34 (sequential order) ------------------ */
void fvo_conservation(int neq, const fvgpu_mesh_soa *m, const double *S, double *sums) {
  const int64_t n = m->ncells;
  for (int v = 0; v <= neq; ++v) sums[v] = 0.0;
  for (int64_t c = 0; c < n; ++c) {
    for (int v = 0; v < neq; ++v) sums[v] += S[(int64_t)v * n + c] * m->vol[c];
    sums[neq] += m->vol[c];
  }
}

/* ---- CFL spectral radius (no reference code; restated definition) -------------------
 * lambda_c = (sum over faces f and sub-faces s of A_s (|u . n_f| + c)) / (2 V_c)
 * with u, c from the cell state (facevalues.c EOS); dt = cfl / max_c lambda_c.
 * For a box cell this equals sum_d (|u_d| + c) / h_d. */
double fvo_cell_lambda(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, int64_t c) {
  const int neq = neq_of(cfg);
  const int64_t n = m->ncells;
  double q[NEQMAX];
  load_cell(U, neq, n, c, q);
  fstate s;
  memset(&s, 0, sizeof s);
  face_state(cfg, q, 0, NULL, &s);
  double acc = 0.0;
  for (int f = 0; f < 6; ++f) {
    const double *fr = m->frames + 9 * f;
    const double un = fabs(s.u * fr[0] + s.v * fr[1] + s.w * fr[2]);
    const int32_t code = m->nbr[(int64_t)f * n + c];
    if (code <= FVGPU_HANG0) {
      const int64_t r = FVGPU_HANG0 - code;
      for (int k = 0; k < 4; ++k) acc += m->hang_area[4 * r + k] * (un + s.c);
    } else {
      acc += m->area[(int64_t)f * n + c] * (un + s.c);
    }
  }
  return acc / (2.0 * m->vol[c]);
}

double fvo_max_lambda(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U) {
  double mx = 0.0;
  for (int64_t c = 0; c < m->ncells; ++c) {
    const double l = fvo_cell_lambda(cfg, m, U, c);
    if (l > mx || isnan(l)) mx = l;
  }
  return mx;
}
