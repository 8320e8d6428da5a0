/*
 * fake_fvgpu.c -- TEST INFRASTRUCTURE ONLY: the subset of include/fvgpu.h
 * that fvshim.c calls, computed on the host by the oracle's C restatement
 * (oracle/fvoracle.c).  Linking the shim against this instead of libfvgpu
 * checks the shim's flattening, state gather / scatter and call mapping on
 * a machine without a GPU, against the reference's own objects.
 */
#include <stdlib.h>
#include <string.h>

#include "fvgpu.h"

/* oracle/fvoracle.c */
void fvo_faceinterp(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, double *SF);
void fvo_gradcalc(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, double *SG);
void fvo_rhs_nb(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const double *U, const double *SF,
                const double *SG, double *R, const int32_t *inner, int inner_outer);
void fvo_rk(int irk, double dt, int neq, const fvgpu_mesh_soa *m, double *S, double *SN, const double *RHS);
void fvo_step(const fvgpu_config *cfg, const fvgpu_mesh_soa *m, const int *stages, int nstages, double dt,
              double *S, double *SN, double *SF, double *SG, double *R);
int fvo_error(int64_t *cell);
void fvo_clear_error(void);

struct fvgpu_ctx {
  fvgpu_config cfg;
  int neq;
  fvgpu_mesh_soa m;
  int32_t *nbr, *nbr_face, *hang_nbr, *level, *inner;
  double *area, *dcf, *dcc, *vol, *hang_area, frames[54];
  double *S, *SN, *R, *SF, *SG;
  int has_sg;
  int calls[16];
};

/* call counters the test reads: 0 faceinterp, 1 gradcalc, 2 rhs, 3 rhs_nb,
 * 4 rk, 5 step, 6 upload_mesh, 7 upload_state, 8 download */
static fvgpu_ctx *g_last;
int fake_calls(int which) { return g_last && which >= 0 && which < 16 ? g_last->calls[which] : -1; }

static void *dup(const void *p, size_t bytes) {
  void *q = malloc(bytes ? bytes : 16);
  if (p && bytes) memcpy(q, p, bytes);
  return q;
}

static int check(fvgpu_ctx *ctx) {
  int64_t cell;
  const int e = fvo_error(&cell);
  fvo_clear_error();
  (void)ctx;
  if (e == 0) return FVGPU_OK;
  return e == 2 ? FVGPU_ERR_EOS : FVGPU_ERR_NONFINITE;
}

int fvgpu_create(const fvgpu_config *cfg, fvgpu_ctx **out) {
  fvgpu_ctx *c = calloc(1, sizeof *c);
  c->cfg = *cfg;
  c->neq = cfg->model == 2 ? 4 : 5;
  *out = c;
  g_last = c;
  return FVGPU_OK;
}

static void release_mesh(fvgpu_ctx *c) {
  free(c->nbr); free(c->nbr_face); free(c->hang_nbr); free(c->level); free(c->inner);
  free(c->area); free(c->dcf); free(c->dcc); free(c->vol); free(c->hang_area);
  free(c->S); free(c->SN); free(c->R); free(c->SF); free(c->SG);
  c->inner = NULL;
}

int fvgpu_destroy(fvgpu_ctx *c) {
  if (!c) return FVGPU_OK;
  release_mesh(c);
  if (g_last == c) g_last = NULL;
  free(c);
  return FVGPU_OK;
}

int fvgpu_set_precision(fvgpu_ctx *c, int precision) {
  c->cfg.precision = precision;
  return FVGPU_OK;
}

int fvgpu_upload_mesh(fvgpu_ctx *c, const fvgpu_mesh_soa *m) {
  release_mesh(c);
  const int64_t n = m->ncells, nh = m->nhang;
  c->nbr = dup(m->nbr, sizeof(int32_t) * 6 * n);
  c->nbr_face = dup(m->nbr_face, sizeof(int32_t) * 6 * n);
  c->area = dup(m->area, sizeof(double) * 6 * n);
  c->dcf = dup(m->dcf, sizeof(double) * 6 * n);
  c->dcc = dup(m->dcc, sizeof(double) * 6 * n);
  c->vol = dup(m->vol, sizeof(double) * n);
  c->hang_nbr = dup(m->hang_nbr, sizeof(int32_t) * 4 * nh);
  c->hang_area = dup(m->hang_area, sizeof(double) * 4 * nh);
  c->level = dup(m->level, sizeof(int32_t) * n);
  memcpy(c->frames, m->frames, sizeof c->frames);
  c->m = *m;
  c->m.nbr = c->nbr;
  c->m.nbr_face = c->nbr_face;
  c->m.area = c->area;
  c->m.dcf = c->dcf;
  c->m.dcc = c->dcc;
  c->m.vol = c->vol;
  c->m.hang_nbr = c->hang_nbr;
  c->m.hang_area = c->hang_area;
  c->m.frames = c->frames;
  c->m.level = c->level;
  const size_t sz = sizeof(double) * (size_t)(c->neq * n);
  c->S = calloc(1, sz);
  c->SN = calloc(1, sz);
  c->R = calloc(1, sz);
  c->SF = calloc(6, sz);
  c->SG = calloc(1, sizeof(double) * (size_t)((c->neq + 1) * 3 * n));
  c->calls[6]++;
  return FVGPU_OK;
}

int fvgpu_upload_state(fvgpu_ctx *c, const double *U, int64_t ld) {
  const int64_t n = c->m.ncells;
  for (int v = 0; v < c->neq; ++v) memcpy(c->S + v * n, U + v * ld, sizeof(double) * (size_t)n);
  c->calls[7]++;
  return FVGPU_OK;
}

int fvgpu_download_state(fvgpu_ctx *c, double *U, int64_t ld) {
  const int64_t n = c->m.ncells;
  for (int v = 0; v < c->neq; ++v) memcpy(U + v * ld, c->S + v * n, sizeof(double) * (size_t)n);
  return FVGPU_OK;
}

int fvgpu_download(fvgpu_ctx *c, int field, double *out) {
  const int64_t n = c->m.ncells;
  const size_t sz = sizeof(double) * (size_t)(c->neq * n);
  c->calls[8]++;
  switch (field) {
    case FVGPU_FIELD_S: memcpy(out, c->S, sz); return FVGPU_OK;
    case FVGPU_FIELD_SN: memcpy(out, c->SN, sz); return FVGPU_OK;
    case FVGPU_FIELD_RHS: memcpy(out, c->R, sz); return FVGPU_OK;
    case FVGPU_FIELD_SF: memcpy(out, c->SF, 6 * sz); return FVGPU_OK;
    case FVGPU_FIELD_SG: memcpy(out, c->SG, sizeof(double) * (size_t)((c->neq + 1) * 3 * n)); return FVGPU_OK;
    default: return FVGPU_ERR_ARG;
  }
}

int fvgpu_faceinterp(fvgpu_ctx *c) {
  fvo_faceinterp(&c->cfg, &c->m, c->S, c->SF);
  c->calls[0]++;
  return check(c);
}

int fvgpu_gradcalc(fvgpu_ctx *c) {
  fvo_gradcalc(&c->cfg, &c->m, c->S, c->SG);
  c->calls[1]++;
  return check(c);
}

int fvgpu_rhs(fvgpu_ctx *c) {
  fvo_rhs_nb(&c->cfg, &c->m, c->S, c->SF, c->SG, c->R, NULL, 0);
  c->calls[2]++;
  return check(c);
}

int fvgpu_set_inner(fvgpu_ctx *c, const int32_t *inner) {
  free(c->inner);
  c->inner = dup(inner, sizeof(int32_t) * (size_t)c->m.ncells);
  return FVGPU_OK;
}

int fvgpu_rhs_nb(fvgpu_ctx *c, int inner_outer) {
  fvo_rhs_nb(&c->cfg, &c->m, c->S, c->SF, c->SG, c->R, c->inner, inner_outer);
  c->calls[3]++;
  return check(c);
}

int fvgpu_rk(fvgpu_ctx *c, int irk, double dt) {
  fvo_rk(irk, dt, c->neq, &c->m, c->S, c->SN, c->R);
  c->calls[4]++;
  return FVGPU_OK;
}

int fvgpu_step(fvgpu_ctx *c, int scheme, double dt, double cfl, int nsteps) {
  static const int kStages[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 4, 0}, {1, 2, 3}};
  (void)cfl;
  if (scheme < 1 || scheme > 3 || !(dt > 0.0)) return FVGPU_ERR_ARG;
  for (int s = 0; s < nsteps; ++s)
    fvo_step(&c->cfg, &c->m, kStages[scheme], scheme, dt, c->S, c->SN, c->SF, c->SG, c->R);
  c->calls[5]++;
  return check(c);
}

int fvgpu_last_error(fvgpu_ctx *c, int *code, int64_t *cell, char *msg, int msglen) {
  (void)c;
  if (code) *code = 0;
  if (cell) *cell = -1;
  if (msg && msglen > 0) strncpy(msg, "oracle error", (size_t)msglen - 1);
  return FVGPU_OK;
}
