/*
 * oracle.c -- CPU oracle for the interval branch-and-bound hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed
 * CPU baseline.  Only tests/, the smoke check and bench.py's CPU arm load
 * it; the product library never does.  Each function cites the reference
 * (CuMINLPSearch) file:line whose behaviour it restates.
 *
 * Build: cc -O2 -std=c11 -ffp-contract=off -fPIC -shared oracle.c -lm
 *        -lpthread
 */
#define _GNU_SOURCE
#include <float.h>
#include <fenv.h>
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ======================================================================
 * errors
 * ==================================================================== */
static __thread char g_err[512];

const char* orc_last_error(void) { return g_err; }

static void set_err(const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

/* ======================================================================
 * directed rounding, double
 * ==================================================================== */
static inline uint64_t dbits(double x)
{
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}
static inline double bitsd(uint64_t u)
{
  double x;
  memcpy(&x, &u, 8);
  return x;
}
static inline double next_up(double x)
{
  if (x != x || x == INFINITY) return x;
  if (x == 0.0) return bitsd(1);
  uint64_t u = dbits(x);
  u = x > 0 ? u + 1 : u - 1;
  return bitsd(u);
}
static inline double next_down(double x) { return -next_up(-x); }

double orc_add_rd(double a, double b)
{
  double s = a + b;
  if (isnan(s)) return s;
  if (isinf(s)) {
    if (isinf(a) || isinf(b)) return s;
    return s > 0 ? DBL_MAX : s;
  }
  if (s == 0.0) /* exact zero: IEEE sign rule of roundTowardNegative */
    return (a == 0.0 && b == 0.0 && !signbit(a) && !signbit(b)) ? 0.0 : -0.0;
  double z = s - a;
  double e = (a - (s - z)) + (b - z);
  return e < 0 ? next_down(s) : s;
}

double orc_add_ru(double a, double b)
{
  double s = a + b;
  if (isnan(s)) return s;
  if (isinf(s)) {
    if (isinf(a) || isinf(b)) return s;
    return s < 0 ? -DBL_MAX : s;
  }
  if (s == 0.0)
    return (a == 0.0 && b == 0.0 && signbit(a) && signbit(b)) ? -0.0 : 0.0;
  double z = s - a;
  double e = (a - (s - z)) + (b - z);
  return e > 0 ? next_up(s) : s;
}

static inline double sub_rd(double a, double b) { return orc_add_rd(a, -b); }
static inline double sub_ru(double a, double b) { return orc_add_ru(a, -b); }

double orc_mul_rd(double a, double b)
{
  double p = a * b;
  if (isnan(p)) return p;
  if (isinf(p)) {
    if (isinf(a) || isinf(b)) return p;
    return p > 0 ? DBL_MAX : p;
  }
  if (p == 0.0) {
    if (a == 0.0 || b == 0.0) return p;
    return signbit(a) != signbit(b) ? -bitsd(1) : 0.0;
  }
  double e = fma(a, b, -p);
  return e < 0 ? next_down(p) : p;
}

double orc_mul_ru(double a, double b)
{
  double p = a * b;
  if (isnan(p)) return p;
  if (isinf(p)) {
    if (isinf(a) || isinf(b)) return p;
    return p < 0 ? -DBL_MAX : p;
  }
  if (p == 0.0) {
    if (a == 0.0 || b == 0.0) return p;
    return signbit(a) != signbit(b) ? -0.0 : bitsd(1);
  }
  double e = fma(a, b, -p);
  return e > 0 ? next_up(p) : p;
}

double orc_div_rd(double a, double b)
{
  double q = a / b;
  if (isnan(q)) return q;
  if (isinf(q)) {
    if (isinf(a) || b == 0.0) return q;
    return q > 0 ? DBL_MAX : q;
  }
  if (q == 0.0) {
    if (a == 0.0 || isinf(b)) return q;
    return signbit(a) != signbit(b) ? -bitsd(1) : 0.0;
  }
  double r = fma(-q, b, a);
  if (r == 0.0) return q;
  return ((r < 0) != (b < 0)) ? next_down(q) : q;
}

double orc_div_ru(double a, double b)
{
  double q = a / b;
  if (isnan(q)) return q;
  if (isinf(q)) {
    if (isinf(a) || b == 0.0) return q;
    return q < 0 ? -DBL_MAX : q;
  }
  if (q == 0.0) {
    if (a == 0.0 || isinf(b)) return q;
    return signbit(a) != signbit(b) ? -0.0 : bitsd(1);
  }
  double r = fma(-q, b, a);
  if (r == 0.0) return q;
  return ((r < 0) == (b < 0)) ? next_up(q) : q;
}

static inline double sqrt_rd(double a)
{
  double s = sqrt(a);
  if (!(s > 0) || isinf(s)) return s;
  double e = fma(s, s, -a);
  return e > 0 ? next_down(s) : s;
}

static inline double sqrt_ru(double a)
{
  double s = sqrt(a);
  if (!(s >= 0) || isinf(s)) return s;
  double e = fma(s, s, -a);
  return e < 0 ? next_up(s) : s;
}

/* ======================================================================
 * directed rounding, float (exact via double arithmetic)
 * ==================================================================== */
static inline uint32_t fbits(float x)
{
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
}
static inline float bitsf(uint32_t u)
{
  float x;
  memcpy(&x, &u, 4);
  return x;
}
static inline float next_upf(float x)
{
  if (x != x || x == INFINITY) return x;
  if (x == 0.0f) return bitsf(1);
  uint32_t u = fbits(x);
  u = x > 0 ? u + 1 : u - 1;
  return bitsf(u);
}
static inline float next_downf(float x) { return -next_upf(-x); }

/* Rounds the exact value s + e (a double-double with |e| <= ulp(s)/2) to a
 * float in the given direction (dir -1 down, +1 up). */
static inline float round_dd_to_float(double s, double e, int dir)
{
  if (isnan(s)) return (float)s;
  float f = (float)s;
  if (isinf(f) && !isinf(s)) f = (s > 0) ? INFINITY : -INFINITY;
  int cmp; /* sign of f - (s + e) */
  if (isinf(f)) {
    cmp = f > 0 ? 1 : -1;
  } else {
    double fd = (double)f;
    if (fd > s) cmp = 1;
    else if (fd < s) cmp = -1;
    else cmp = e < 0 ? 1 : (e > 0 ? -1 : 0);
  }
  if (dir < 0) {
    if (cmp > 0) {
      if (f == INFINITY) return FLT_MAX;
      return next_downf(f);
    }
    return f;
  }
  if (cmp < 0) {
    if (f == -INFINITY) return -FLT_MAX;
    return next_upf(f);
  }
  return f;
}

static inline float addf_dir(float a, float b, int dir)
{
  if (isinf(a) || isinf(b) || isnan(a) || isnan(b)) return a + b;
  double A = a, B = b;
  double s = A + B;
  if (s == 0.0) {
    if (dir < 0) return (a == 0.0f && b == 0.0f && !signbit(a) && !signbit(b)) ? 0.0f : -0.0f;
    return (a == 0.0f && b == 0.0f && signbit(a) && signbit(b)) ? -0.0f : 0.0f;
  }
  double z = s - A;
  double e = (A - (s - z)) + (B - z);
  return round_dd_to_float(s, e, dir);
}

float orc_addf_rd(float a, float b) { return addf_dir(a, b, -1); }
float orc_addf_ru(float a, float b) { return addf_dir(a, b, +1); }
static inline float subf_rd(float a, float b) { return addf_dir(a, -b, -1); }
static inline float subf_ru(float a, float b) { return addf_dir(a, -b, +1); }

static inline float mulf_dir(float a, float b, int dir)
{
  if (isinf(a) || isinf(b) || isnan(a) || isnan(b)) return a * b;
  double p = (double)a * (double)b; /* exact: 24+24 bits */
  if (p == 0.0) return a * b;        /* exact zero, IEEE sign */
  return round_dd_to_float(p, 0.0, dir);
}

float orc_mulf_rd(float a, float b) { return mulf_dir(a, b, -1); }
float orc_mulf_ru(float a, float b) { return mulf_dir(a, b, +1); }

static inline float divf_dir(float a, float b, int dir)
{
  float q = a / b;
  if (isnan(q)) return q;
  if (isinf(q)) {
    if (isinf(a) || b == 0.0f) return q;
    if (dir < 0) return q > 0 ? FLT_MAX : q;
    return q < 0 ? -FLT_MAX : q;
  }
  if (q == 0.0f) {
    if (a == 0.0f || isinf(b)) return q;
    if (dir < 0) return signbit(a) != signbit(b) ? -bitsf(1) : 0.0f;
    return signbit(a) != signbit(b) ? -0.0f : bitsf(1);
  }
  /* exact remainder a - q*b, computed in double (q*b exact in double) */
  double r = (double)a - (double)q * (double)b;
  if (r == 0.0) return q;
  int too_big = (r < 0) != (b < 0); /* true quotient below q */
  if (dir < 0) return too_big ? next_downf(q) : q;
  return too_big ? q : next_upf(q);
}

static inline float divf_rd(float a, float b) { return divf_dir(a, b, -1); }
static inline float divf_ru(float a, float b) { return divf_dir(a, b, +1); }

static inline float sqrtf_dir(float a, int dir)
{
  float s = sqrtf(a);
  if (!(s > 0) || isinf(s)) return s;
  double sq = (double)s * (double)s; /* exact */
  if (dir < 0) return sq > (double)a ? next_downf(s) : s;
  return sq < (double)a ? next_upf(s) : s;
}

static inline float sqrtf_rd(float a) { return sqrtf_dir(a, -1); }
static inline float sqrtf_ru(float a) { return sqrtf_dir(a, +1); }

float orc_d2f_rd(double a)
{
  if (isnan(a)) return (float)a;
  float f = (float)a;
  if (isinf(f) && !isinf(a)) return a > 0 ? FLT_MAX : -INFINITY;
  return (double)f > a ? next_downf(f) : f;
}

float orc_d2f_ru(double a)
{
  if (isnan(a)) return (float)a;
  float f = (float)a;
  if (isinf(f) && !isinf(a)) return a < 0 ? -FLT_MAX : INFINITY;
  return (double)f < a ? next_upf(f) : f;
}

/* ======================================================================
 * interval operators (tightest enclosures), double and float
 * ==================================================================== */
typedef struct { double lo, hi; } iv64;
typedef struct { float lo, hi; } iv32;

#define T double
#define IV iv64
#define SUF(n) n##_d
#define ADD_RD orc_add_rd
#define ADD_RU orc_add_ru
#define SUB_RD sub_rd
#define SUB_RU sub_ru
#define MUL_RD orc_mul_rd
#define MUL_RU orc_mul_ru
#define DIV_RD orc_div_rd
#define DIV_RU orc_div_ru
#define SQRT_RD sqrt_rd
#define SQRT_RU sqrt_ru
#define T_INF INFINITY
#include "oracle_interval.inc"
#undef T
#undef IV
#undef SUF
#undef ADD_RD
#undef ADD_RU
#undef SUB_RD
#undef SUB_RU
#undef MUL_RD
#undef MUL_RU
#undef DIV_RD
#undef DIV_RU
#undef SQRT_RD
#undef SQRT_RU
#undef T_INF

#define T float
#define IV iv32
#define SUF(n) n##_f
#define ADD_RD orc_addf_rd
#define ADD_RU orc_addf_ru
#define SUB_RD subf_rd
#define SUB_RU subf_ru
#define MUL_RD orc_mulf_rd
#define MUL_RU orc_mulf_ru
#define DIV_RD divf_rd
#define DIV_RU divf_ru
#define SQRT_RD sqrtf_rd
#define SQRT_RU sqrtf_ru
#define T_INF INFINITY
#include "oracle_interval.inc"
#undef T
#undef IV
#undef SUF
#undef ADD_RD
#undef ADD_RU
#undef SUB_RD
#undef SUB_RU
#undef MUL_RD
#undef MUL_RU
#undef DIV_RD
#undef DIV_RU
#undef SQRT_RD
#undef SQRT_RU
#undef T_INF

/* The same operators with the host's directed-rounding hardware, for the
 * timed CPU path of the bench: the calling thread's rounding mode is
 * FE_DOWNWARD for a whole box evaluation, so round-down results are the
 * plain IEEE operations and round-up ones are negated round-down ones
 * (ru(x op y) = -rd(-(x op y))).  Tested bit for bit against the error-free
 * transformations above.  Sqrt (whose round-up form has no such identity)
 * and the remaining operators run through the software forms under
 * round-to-nearest (apply_hw). */
static inline double hw_add_ru(double a, double b) { return -((-a) + (-b)); }
static inline double hw_sub_ru(double a, double b) { return -(b - a); }
static inline double hw_mul_ru(double a, double b) { return -((-a) * b); }
static inline double hw_div_ru(double a, double b) { return -((-a) / b); }
static inline double hw_add_rd(double a, double b) { return a + b; }
static inline double hw_sub_rd(double a, double b) { return a - b; }
static inline double hw_mul_rd(double a, double b) { return a * b; }
static inline double hw_div_rd(double a, double b) { return a / b; }

#define T double
#define IV iv64
#define SUF(n) n##_h
#define ADD_RD hw_add_rd
#define ADD_RU hw_add_ru
#define SUB_RD hw_sub_rd
#define SUB_RU hw_sub_ru
#define MUL_RD hw_mul_rd
#define MUL_RU hw_mul_ru
#define DIV_RD hw_div_rd
#define DIV_RU hw_div_ru
#define SQRT_RD sqrt_rd
#define SQRT_RU sqrt_ru
#define T_INF INFINITY
#include "oracle_interval.inc"
#undef T
#undef IV
#undef SUF
#undef ADD_RD
#undef ADD_RU
#undef SUB_RD
#undef SUB_RU
#undef MUL_RD
#undef MUL_RU
#undef DIV_RD
#undef DIV_RU
#undef SQRT_RD
#undef SQRT_RU
#undef T_INF

static int op_supported_interval(int op)
{
  switch (op) {
    case CMN_OP_VAR: case CMN_OP_CONST: case CMN_OP_ADD: case CMN_OP_SUB:
    case CMN_OP_MUL: case CMN_OP_DIV: case CMN_OP_SQR: case CMN_OP_NEG:
    case CMN_OP_SQRT: case CMN_OP_POWN: case CMN_OP_ABS: case CMN_OP_MIN:
    case CMN_OP_MAX:
      return 1;
    default:
      return 0;
  }
}

static iv64 apply_d(int op, iv64 a, iv64 b, int k)
{
  switch (op) {
    case CMN_OP_ADD: return iv_add_d(a, b);
    case CMN_OP_SUB: return iv_sub_d(a, b);
    case CMN_OP_MUL: return iv_mul_d(a, b);
    case CMN_OP_DIV: return iv_div_d(a, b);
    case CMN_OP_SQR: return iv_sqr_d(a);
    case CMN_OP_NEG: return iv_neg_d(a);
    case CMN_OP_SQRT: return iv_sqrt_d(a);
    case CMN_OP_POWN: return iv_pown_d(a, k);
    case CMN_OP_ABS: return iv_abs_d(a);
    case CMN_OP_MIN: return iv_min_d(a, b);
    case CMN_OP_MAX: return iv_max_d(a, b);
    default: {
      iv64 r = {NAN, NAN};
      return r;
    }
  }
}

/* under FE_DOWNWARD (see the _h operators) */
static iv64 apply_hw(int op, iv64 a, iv64 b, int k)
{
  switch (op) {
    case CMN_OP_ADD: return iv_add_h(a, b);
    case CMN_OP_SUB: return iv_sub_h(a, b);
    case CMN_OP_MUL: return iv_mul_h(a, b);
    case CMN_OP_DIV: return iv_div_h(a, b);
    case CMN_OP_SQR: return iv_sqr_h(a);
    case CMN_OP_NEG: return iv_neg_h(a);
    default: {
      fesetround(FE_TONEAREST);
      iv64 r = apply_d(op, a, b, k);
      fesetround(FE_DOWNWARD);
      return r;
    }
  }
}

static iv32 apply_f(int op, iv32 a, iv32 b, int k)
{
  switch (op) {
    case CMN_OP_ADD: return iv_add_f(a, b);
    case CMN_OP_SUB: return iv_sub_f(a, b);
    case CMN_OP_MUL: return iv_mul_f(a, b);
    case CMN_OP_DIV: return iv_div_f(a, b);
    case CMN_OP_SQR: return iv_sqr_f(a);
    case CMN_OP_NEG: return iv_neg_f(a);
    case CMN_OP_SQRT: return iv_sqrt_f(a);
    case CMN_OP_POWN: return iv_pown_f(a, k);
    case CMN_OP_ABS: return iv_abs_f(a);
    case CMN_OP_MIN: return iv_min_f(a, b);
    case CMN_OP_MAX: return iv_max_f(a, b);
    default: {
      iv32 r = {NAN, NAN};
      return r;
    }
  }
}

void orc_interval_op_f64(int op, double alo, double ahi, double blo,
                         double bhi, int int_exp, double* lo, double* hi)
{
  iv64 a = {alo, ahi}, b = {blo, bhi};
  iv64 r = apply_d(op, a, b, int_exp);
  *lo = r.lo;
  *hi = r.hi;
}

void orc_interval_op_f32(int op, float alo, float ahi, float blo, float bhi,
                         int int_exp, float* lo, float* hi)
{
  iv32 a = {alo, ahi}, b = {blo, bhi};
  iv32 r = apply_f(op, a, b, int_exp);
  *lo = r.lo;
  *hi = r.hi;
}

/* Point operators: plain round-to-nearest T arithmetic, one rounding per
 * DAG node (graph/ops.cuh point overloads; graph/kernels.cuh:177-281 run one
 * kernel per node, so nothing contracts across nodes). */
static double point_apply(int op, double a, double b, int k)
{
  switch (op) {
    case CMN_OP_ADD: return a + b;
    case CMN_OP_SUB: return a - b;
    case CMN_OP_MUL: return a * b;
    case CMN_OP_DIV: return a / b;
    case CMN_OP_SQR: return a * a;
    case CMN_OP_NEG: return -a;
    case CMN_OP_EXP: return exp(a);
    case CMN_OP_LOG: return log(a);
    case CMN_OP_SQRT: return sqrt(a);
    case CMN_OP_SIN: return sin(a);
    case CMN_OP_COS: return cos(a);
    case CMN_OP_TANH: return tanh(a);
    case CMN_OP_POWN: return pow(a, (double)k);
    case CMN_OP_POW: return pow(a, b);
    case CMN_OP_ABS: return fabs(a);
    case CMN_OP_MIN: return fmin(a, b);
    case CMN_OP_MAX: return fmax(a, b);
    default: return NAN;
  }
}

/* ======================================================================
 * problem
 * ==================================================================== */
struct orc_problem {
  int64_t n_nodes, n_vars, n_cons, root;
  cmn_node* nodes;
  double* var_lb;
  double* var_ub;
  int32_t* kinds;
  cmn_constraint* cons;
  uint8_t* reach; /* reachable from a root (backend/graph/cost.hpp:38-68) */
  int64_t n_reach;
  int64_t* order; /* reachable non-Const, non-Var node ids, ascending */
  int64_t n_order;
  float* clo32; /* per node: FP32 outward bounds of a Const payload */
  float* chi32;
  /* the lazy form's incremental FP32 children (orc_set_program32) */
  int inc_ok;
  int64_t prog_len;
  struct orc_instr* prog32;
  struct orc_instr* prog64; /* the FP64 program: the lazy form's fused verdict */
  int64_t prog64_len;
  int64_t n_prog_slots;
  int64_t inc_segments;
  int32_t* inc_seg; /* 3 per segment: chain [b, t), checks/objective [t, e) */
  int32_t* inc_off; /* n_vars * segments + 1 */
  int32_t* inc_pcs;
};

void orc_problem_destroy(orc_problem* p)
{
  if (!p) return;
  free(p->nodes);
  free(p->var_lb);
  free(p->var_ub);
  free(p->kinds);
  free(p->cons);
  free(p->reach);
  free(p->order);
  free(p->clo32);
  free(p->chi32);
  free(p->prog32);
  free(p->prog64);
  free(p->inc_seg);
  free(p->inc_off);
  free(p->inc_pcs);
  free(p);
}

static int is_unary(int op)
{
  return op == CMN_OP_SQR || op == CMN_OP_NEG || op == CMN_OP_EXP ||
         op == CMN_OP_LOG || op == CMN_OP_SQRT || op == CMN_OP_SIN ||
         op == CMN_OP_COS || op == CMN_OP_TANH || op == CMN_OP_POWN ||
         op == CMN_OP_ABS;
}

orc_problem* orc_problem_create(const cmn_problem_desc* d)
{
  if (!d || d->n_nodes <= 0 || !d->nodes) {
    set_err("empty DAG");
    return NULL;
  }
  orc_problem* p = (orc_problem*)calloc(1, sizeof *p);
  p->n_nodes = d->n_nodes;
  p->n_vars = d->n_vars;
  p->n_cons = d->n_constraints;
  p->root = d->objective_root;
  p->nodes = (cmn_node*)malloc(sizeof(cmn_node) * (size_t)d->n_nodes);
  memcpy(p->nodes, d->nodes, sizeof(cmn_node) * (size_t)d->n_nodes);
  size_t nv = (size_t)(d->n_vars > 0 ? d->n_vars : 1);
  p->var_lb = (double*)malloc(sizeof(double) * nv);
  p->var_ub = (double*)malloc(sizeof(double) * nv);
  p->kinds = (int32_t*)malloc(sizeof(int32_t) * nv);
  if (d->n_vars > 0) {
    memcpy(p->var_lb, d->var_lb, sizeof(double) * (size_t)d->n_vars);
    memcpy(p->var_ub, d->var_ub, sizeof(double) * (size_t)d->n_vars);
    memcpy(p->kinds, d->var_kinds, sizeof(int32_t) * (size_t)d->n_vars);
  }
  size_t nc = (size_t)(d->n_constraints > 0 ? d->n_constraints : 1);
  p->cons = (cmn_constraint*)malloc(sizeof(cmn_constraint) * nc);
  if (d->n_constraints > 0)
    memcpy(p->cons, d->constraints, sizeof(cmn_constraint) * (size_t)d->n_constraints);

  /* structural checks of Problem::validate (model/problem.hpp:282-355) */
  int64_t n_var_nodes = 0;
  for (int64_t i = 0; i < p->n_nodes; ++i) {
    const cmn_node* nd = &p->nodes[i];
    if (nd->op < 0 || nd->op > CMN_OP_MAX) {
      set_err("node %lld has an unknown op", (long long)i);
      goto fail;
    }
    int need = (nd->op == CMN_OP_VAR || nd->op == CMN_OP_CONST) ? 0 : (is_unary(nd->op) ? 1 : 2);
    if (nd->n_in != need) {
      set_err("node %lld has %d operands, op needs %d", (long long)i, nd->n_in, need);
      goto fail;
    }
    if ((need >= 1 && (nd->in0 < 0 || nd->in0 >= i)) || (need >= 2 && (nd->in1 < 0 || nd->in1 >= i))) {
      set_err("DAG node operand id is not strictly less than the node's own id");
      goto fail;
    }
    if (nd->op == CMN_OP_VAR) {
      if (nd->var_index != n_var_nodes) {
        set_err("Var node var_index out of order");
        goto fail;
      }
      ++n_var_nodes;
    }
  }
  if (n_var_nodes != p->n_vars) {
    set_err("box_bounds/var_kinds are out of sync with the number of Op::Var nodes");
    goto fail;
  }
  if (p->n_vars == 0) {
    set_err("Problem has zero variables");
    goto fail;
  }
  if (p->root < 0 || p->root >= p->n_nodes) {
    set_err("Problem's objective was never set");
    goto fail;
  }
  if (p->nodes[p->root].op == CMN_OP_CONST) {
    set_err("objective root is a bare Const");
    goto fail;
  }
  for (int64_t c = 0; c < p->n_cons; ++c) {
    if (p->cons[c].root < 0 || p->cons[c].root >= p->n_nodes) {
      set_err("constraint root out of range");
      goto fail;
    }
    if (p->nodes[p->cons[c].root].op == CMN_OP_CONST) {
      set_err("constraint root is a bare Const");
      goto fail;
    }
    if (!isfinite(p->cons[c].rhs)) {
      set_err("constraint rhs must be finite");
      goto fail;
    }
  }
  for (int64_t v = 0; v < p->n_vars; ++v) {
    double lb = p->var_lb[v], ub = p->var_ub[v];
    if (!(lb <= ub)) {
      set_err("variable's lower bound exceeds its upper bound");
      goto fail;
    }
    if (p->kinds[v] == CMN_VAR_INTEGER || p->kinds[v] == CMN_VAR_BINARY) {
      if (floor(lb) < lb || floor(ub) < ub) {
        set_err("Integer/Binary variable has non-integer-valued bounds");
        goto fail;
      }
    }
    if (p->kinds[v] == CMN_VAR_BINARY && (lb < 0 || lb > 0 || ub < 1 || ub > 1)) {
      set_err("Binary variable's bounds are not exactly [0,1]");
      goto fail;
    }
  }

  /* reachability (backend/graph/cost.hpp:38-68) */
  p->reach = (uint8_t*)calloc((size_t)p->n_nodes, 1);
  p->reach[p->root] = 1;
  for (int64_t c = 0; c < p->n_cons; ++c) p->reach[p->cons[c].root] = 1;
  for (int64_t i = p->n_nodes - 1; i >= 0; --i) {
    if (!p->reach[i]) continue;
    const cmn_node* nd = &p->nodes[i];
    if (nd->n_in >= 1) p->reach[nd->in0] = 1;
    if (nd->n_in >= 2) p->reach[nd->in1] = 1;
  }
  p->order = (int64_t*)malloc(sizeof(int64_t) * (size_t)p->n_nodes);
  p->n_order = 0;
  p->n_reach = 0;
  for (int64_t i = 0; i < p->n_nodes; ++i) {
    if (!p->reach[i]) continue;
    const cmn_node* nd = &p->nodes[i];
    if (nd->op != CMN_OP_CONST) ++p->n_reach;
    if (nd->op == CMN_OP_VAR || nd->op == CMN_OP_CONST) continue;
    if (is_unary(nd->op) && p->nodes[nd->in0].op == CMN_OP_CONST) {
      set_err("unary op applied directly to an Op::Const");
      goto fail;
    }
    p->order[p->n_order++] = i;
  }
  p->clo32 = (float*)malloc(sizeof(float) * (size_t)p->n_nodes);
  p->chi32 = (float*)malloc(sizeof(float) * (size_t)p->n_nodes);
  for (int64_t i = 0; i < p->n_nodes; ++i) {
    double c = p->nodes[i].constant;
    p->clo32[i] = orc_d2f_rd(c);
    p->chi32[i] = orc_d2f_ru(c);
  }
  return p;
fail:
  orc_problem_destroy(p);
  return NULL;
}

int64_t orc_buffer_node_count(const orc_problem* p) { return p->n_reach; }

/* ======================================================================
 * interval DAG evaluation (one value per node, graph/kernels.cuh:177-281)
 * ==================================================================== */
static int eval_all_d(const orc_problem* p, const double* box, iv64* val)
{
  for (int64_t v = 0; v < p->n_nodes; ++v) {
    const cmn_node* nd = &p->nodes[v];
    if (nd->op == CMN_OP_VAR && p->reach[v]) {
      val[v].lo = box[2 * nd->var_index];
      val[v].hi = box[2 * nd->var_index + 1];
    } else if (nd->op == CMN_OP_CONST) {
      val[v].lo = nd->constant;
      val[v].hi = nd->constant;
    }
  }
  for (int64_t k = 0; k < p->n_order; ++k) {
    int64_t i = p->order[k];
    const cmn_node* nd = &p->nodes[i];
    if (!op_supported_interval(nd->op)) return -1;
    iv64 a = val[nd->in0];
    iv64 b = nd->n_in >= 2 ? val[nd->in1] : a;
    val[i] = apply_d(nd->op, a, b, nd->int_exp);
  }
  return 0;
}

/* eval_all_d with the hardware operators; the caller has set FE_DOWNWARD */
static int eval_all_hw(const orc_problem* p, const double* box, iv64* val)
{
  for (int64_t v = 0; v < p->n_nodes; ++v) {
    const cmn_node* nd = &p->nodes[v];
    if (nd->op == CMN_OP_VAR && p->reach[v]) {
      val[v].lo = box[2 * nd->var_index];
      val[v].hi = box[2 * nd->var_index + 1];
    } else if (nd->op == CMN_OP_CONST) {
      val[v].lo = nd->constant;
      val[v].hi = nd->constant;
    }
  }
  for (int64_t k = 0; k < p->n_order; ++k) {
    int64_t i = p->order[k];
    const cmn_node* nd = &p->nodes[i];
    if (!op_supported_interval(nd->op)) return -1;
    iv64 a = val[nd->in0];
    iv64 b = nd->n_in >= 2 ? val[nd->in1] : a;
    val[i] = apply_hw(nd->op, a, b, nd->int_exp);
  }
  return 0;
}

static int eval_all_f(const orc_problem* p, const double* box, iv32* val)
{
  for (int64_t v = 0; v < p->n_nodes; ++v) {
    const cmn_node* nd = &p->nodes[v];
    if (nd->op == CMN_OP_VAR && p->reach[v]) {
      val[v].lo = orc_d2f_rd(box[2 * nd->var_index]);
      val[v].hi = orc_d2f_ru(box[2 * nd->var_index + 1]);
    } else if (nd->op == CMN_OP_CONST) {
      val[v].lo = p->clo32[v];
      val[v].hi = p->chi32[v];
    }
  }
  for (int64_t k = 0; k < p->n_order; ++k) {
    int64_t i = p->order[k];
    const cmn_node* nd = &p->nodes[i];
    if (!op_supported_interval(nd->op)) return -1;
    iv32 a = val[nd->in0];
    iv32 b = nd->n_in >= 2 ? val[nd->in1] : a;
    val[i] = apply_f(nd->op, a, b, nd->int_exp);
  }
  return 0;
}

int orc_eval_nodes_f64(const orc_problem* p, const double* box,
                       double* node_lo, double* node_hi)
{
  iv64* val = (iv64*)malloc(sizeof(iv64) * (size_t)p->n_nodes);
  int rc = eval_all_d(p, box, val);
  for (int64_t i = 0; i < p->n_nodes; ++i) {
    int keep = p->reach[i] && p->nodes[i].op != CMN_OP_CONST;
    node_lo[i] = keep ? val[i].lo : NAN;
    node_hi[i] = keep ? val[i].hi : NAN;
  }
  free(val);
  if (rc) set_err("op without an interval implementation");
  return rc;
}

int orc_eval_nodes_f32(const orc_problem* p, const double* box,
                       float* node_lo, float* node_hi)
{
  iv32* val = (iv32*)malloc(sizeof(iv32) * (size_t)p->n_nodes);
  int rc = eval_all_f(p, box, val);
  for (int64_t i = 0; i < p->n_nodes; ++i) {
    int keep = p->reach[i] && p->nodes[i].op != CMN_OP_CONST;
    node_lo[i] = keep ? val[i].lo : NAN;
    node_hi[i] = keep ? val[i].hi : NAN;
  }
  free(val);
  if (rc) set_err("op without an interval implementation");
  return rc;
}

/* FP64 verdict of one box: interval feasibility (graph/kernels.cuh:283-306
 * is_feasible for intervals) and objective bounds (kernels.cuh:373-401). */
static int verdict_d(const orc_problem* p, const iv64* val, double* lb,
                     double* ub)
{
  int feas = 1;
  for (int64_t c = 0; c < p->n_cons; ++c) {
    iv64 v = val[p->cons[c].root];
    double rhs = p->cons[c].rhs;
    int ok = p->cons[c].cmp == CMN_CMP_LE ? (v.lo <= rhs)
                                          : (v.lo <= rhs && rhs <= v.hi);
    if (!ok) feas = 0;
  }
  *lb = val[p->root].lo;
  *ub = val[p->root].hi;
  return feas;
}

/* FP32 screen verdict: a box is excluded only when the FP32 enclosure
 * proves it (NaN never excludes), so the FP64 certify pass decides
 * everything the screen leaves open. */
static int verdict_f(const orc_problem* p, const iv32* val, double* lb,
                     double* ub)
{
  int feas = 1;
  for (int64_t c = 0; c < p->n_cons; ++c) {
    iv32 v = val[p->cons[c].root];
    double rhs = p->cons[c].rhs;
    int excluded = p->cons[c].cmp == CMN_CMP_LE
                       ? ((double)v.lo > rhs)
                       : ((double)v.lo > rhs || (double)v.hi < rhs);
    if (excluded) feas = 0;
  }
  *lb = (double)val[p->root].lo;
  *ub = (double)val[p->root].hi;
  return feas;
}

/* ======================================================================
 * tiny pthread parallel-for
 * ==================================================================== */
typedef void (*range_fn)(void* ctx, int64_t begin, int64_t end, int tid);
typedef struct {
  range_fn fn;
  void* ctx;
  int64_t begin, end;
  int tid;
} range_job;

static void* range_thread(void* arg)
{
  range_job* j = (range_job*)arg;
  j->fn(j->ctx, j->begin, j->end, j->tid);
  return NULL;
}

static void parallel_for(int64_t n, int threads, range_fn fn, void* ctx)
{
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  /* a thread start costs tens of microseconds: keep >= 64 items each */
  if (n < 64 * (int64_t)threads) threads = (int)(n / 64 > 0 ? n / 64 : 1);
  if (threads <= 1) {
    fn(ctx, 0, n, 0);
    return;
  }
  pthread_t th[256];
  range_job jobs[256];
  int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].begin = t * chunk;
    jobs[t].end = (t + 1) * chunk < n ? (t + 1) * chunk : n;
    jobs[t].tid = t;
    if (jobs[t].begin >= jobs[t].end) jobs[t].begin = jobs[t].end = n;
    pthread_create(&th[t], NULL, range_thread, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
}

/* ======================================================================
 * batch evaluation over SoA planes
 * ==================================================================== */
typedef struct {
  const orc_problem* p;
  int precision;
  const double *lo, *hi;
  int64_t stride;
  double *obj_lb, *obj_ub;
  uint8_t* feas;
  int failed;
} eval_ctx;

static void eval_range(void* vctx, int64_t b0, int64_t b1, int tid)
{
  (void)tid;
  eval_ctx* c = (eval_ctx*)vctx;
  const orc_problem* p = c->p;
  double* box = (double*)malloc(sizeof(double) * 2 * (size_t)p->n_vars);
  iv64* v64 = (iv64*)malloc(sizeof(iv64) * (size_t)p->n_nodes);
  iv32* v32 = (iv32*)malloc(sizeof(iv32) * (size_t)p->n_nodes);
  for (int64_t b = b0; b < b1; ++b) {
    for (int64_t v = 0; v < p->n_vars; ++v) {
      box[2 * v] = c->lo[v * c->stride + b];
      box[2 * v + 1] = c->hi[v * c->stride + b];
    }
    double lb, ub;
    int f;
    if (c->precision == CMN_PRECISION_FP32_SCREEN) {
      if (eval_all_f(p, box, v32)) c->failed = 1;
      f = verdict_f(p, v32, &lb, &ub);
    } else {
      if (eval_all_d(p, box, v64)) c->failed = 1;
      f = verdict_d(p, v64, &lb, &ub);
    }
    if (c->obj_lb) c->obj_lb[b] = lb;
    if (c->obj_ub) c->obj_ub[b] = ub;
    if (c->feas) c->feas[b] = (uint8_t)f;
  }
  free(box);
  free(v64);
  free(v32);
}

int orc_eval_boxes(const orc_problem* p, int precision, const double* lo,
                   const double* hi, int64_t n_boxes, int64_t stride,
                   double* obj_lb, double* obj_ub, uint8_t* feasible,
                   int threads)
{
  eval_ctx c = {p, precision, lo, hi, stride, obj_lb, obj_ub, feasible, 0};
  parallel_for(n_boxes, threads, eval_range, &c);
  if (c.failed) {
    set_err("op without an interval implementation");
    return -1;
  }
  return 0;
}

/* ======================================================================
 * point evaluation and point feasibility (graph/kernels.cuh:283-320)
 * ==================================================================== */
static int almost_equal(double a, double b)
{
  double diff = fabs(a - b);
  if (diff <= 1e-8) return 1;
  return diff <= 1e-6 * fmax(fabs(a), fabs(b));
}

static int eval_point_impl(const orc_problem* p, const double* x, double* val,
                           double* obj)
{
  for (int64_t v = 0; v < p->n_nodes; ++v) {
    const cmn_node* nd = &p->nodes[v];
    if (nd->op == CMN_OP_VAR) val[v] = x[nd->var_index];
    else if (nd->op == CMN_OP_CONST) val[v] = nd->constant;
  }
  for (int64_t k = 0; k < p->n_order; ++k) {
    int64_t i = p->order[k];
    const cmn_node* nd = &p->nodes[i];
    double a = val[nd->in0];
    double b = nd->n_in >= 2 ? val[nd->in1] : a;
    val[i] = point_apply(nd->op, a, b, nd->int_exp);
  }
  int feas = 1;
  for (int64_t c = 0; c < p->n_cons; ++c) {
    double v = val[p->cons[c].root];
    double rhs = p->cons[c].rhs;
    int ok = p->cons[c].cmp == CMN_CMP_LE ? (v <= rhs) : almost_equal(v, rhs);
    if (!ok) feas = 0;
  }
  *obj = val[p->root];
  return feas;
}

int orc_eval_point(const orc_problem* p, const double* x, double* obj,
                   uint8_t* feasible)
{
  double* val = (double*)malloc(sizeof(double) * (size_t)p->n_nodes);
  *feasible = (uint8_t)eval_point_impl(p, x, val, obj);
  free(val);
  return 0;
}

/* Lazy form's sample screen: FP32 point evaluation, one round-to-nearest
 * float operation per node, the point's variables and the constants
 * rounded to nearest float; constraints by the point predicates on the
 * float values widened to double.  PowN is binary powering (k < 0:
 * 1 / x^|k|).  Restates point_range32 (csrc/eval_core.cuh). */
static float powu_f(float a, int k)
{
  float r = 1.0f, b = a;
  while (k > 0) {
    if (k & 1) r = r * b;
    k >>= 1;
    if (k > 0) b = b * b;
  }
  return r;
}

static float point_apply_f(int op, float a, float b, int k)
{
  switch (op) {
    case CMN_OP_ADD: return a + b;
    case CMN_OP_SUB: return a - b;
    case CMN_OP_MUL: return a * b;
    case CMN_OP_DIV: return a / b;
    case CMN_OP_SQR: return a * a;
    case CMN_OP_NEG: return -a;
    case CMN_OP_SQRT: return sqrtf(a);
    case CMN_OP_POWN: return k == 0 ? 1.0f : (k > 0 ? powu_f(a, k) : 1.0f / powu_f(a, -k));
    case CMN_OP_ABS: return fabsf(a);
    case CMN_OP_MIN: return fminf(a, b);
    case CMN_OP_MAX: return fmaxf(a, b);
    default: return NAN;
  }
}

static int eval_point_f(const orc_problem* p, const double* x, float* val, float* obj)
{
  for (int64_t v = 0; v < p->n_nodes; ++v) {
    const cmn_node* nd = &p->nodes[v];
    if (nd->op == CMN_OP_VAR) val[v] = (float)x[nd->var_index];
    else if (nd->op == CMN_OP_CONST) val[v] = (float)nd->constant;
  }
  for (int64_t k = 0; k < p->n_order; ++k) {
    int64_t i = p->order[k];
    const cmn_node* nd = &p->nodes[i];
    float a = val[nd->in0];
    float b = nd->n_in >= 2 ? val[nd->in1] : a;
    val[i] = point_apply_f(nd->op, a, b, nd->int_exp);
  }
  int feas = 1;
  for (int64_t c = 0; c < p->n_cons; ++c) {
    double v = (double)val[p->cons[c].root];
    double rhs = p->cons[c].rhs;
    int ok = p->cons[c].cmp == CMN_CMP_LE ? (v <= rhs) : almost_equal(v, rhs);
    if (!ok) feas = 0;
  }
  *obj = val[p->root];
  return feas;
}

/* ======================================================================
 * region decode (region/decode.hpp:44-71) and sampler
 * (graph/subregion_sampler.cuh:53-120)
 * ==================================================================== */
/* The device decode is compiled with FMA contraction, so
 * `parent.lb + width * part` is fma(width, part, parent.lb); this oracle
 * states that form explicitly. */
void orc_slot_bounds(int kind, double plo, double phi, uint64_t part,
                     uint64_t fan_out, double* lo, double* hi)
{
  if (kind == CMN_SLOT_INTEGER_ENUMERATE || kind == CMN_SLOT_BINARY_ENUMERATE) {
    double l = ceil(plo);
    double value = l + (double)part;
    if (value > phi) value = phi;
    *lo = value;
    *hi = value;
    return;
  }
  double width = (phi - plo) / (double)fan_out;
  *lo = fma(width, (double)part, plo);
  *hi = (part + 1 == fan_out) ? phi : fma(width, (double)(part + 1), plo);
}

uint64_t orc_sample_hash(uint64_t vid, uint64_t i, uint64_t region,
                         uint64_t salt)
{
  uint64_t x = vid * 0x9e3779b97f4a7c15ULL;
  x ^= i * 0xbf58476d1ce4e5b9ULL;
  x ^= region * 0x94d049bb133111ebULL;
  x ^= salt * 0xd6e8feb86659fd93ULL;
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}

double orc_sample_continuous(double lb, double ub, uint64_t vid, uint64_t i,
                             uint64_t region, uint64_t salt)
{
  uint64_t x = orc_sample_hash(vid, i, region, salt);
  double u = (double)(x >> 11) * (1.0 / 9007199254740992.0);
  return fma(u, ub - lb, lb);
}

double orc_sample_discrete(double lb, double ub, uint64_t vid, uint64_t i,
                           uint64_t region, uint64_t salt)
{
  uint64_t x = orc_sample_hash(vid, i, region, salt);
  double lo = ceil(lb), hi = floor(ub);
  if (hi < lo) return lo;
  uint64_t count = (uint64_t)(hi - lo) + 1;
  uint64_t idx = x % count;
  return lo + (double)idx;
}

float orc_sample_continuous_f32(float lb, float ub, uint64_t vid, uint64_t i,
                                uint64_t region, uint64_t salt)
{
  uint64_t x = orc_sample_hash(vid, i, region, salt);
  float u = (float)(uint32_t)x * (1.0f / 4294967296.0f);
  return fmaf(u, ub - lb, lb);
}

float orc_sample_discrete_f32(float lb, float ub, uint64_t vid, uint64_t i,
                              uint64_t region, uint64_t salt)
{
  uint64_t x = orc_sample_hash(vid, i, region, salt);
  float lo = ceilf(lb), hi = floorf(ub);
  if (hi < lo) return lo;
  uint64_t count = (uint64_t)(hi - lo) + 1;
  uint64_t idx = x % count;
  return lo + (float)idx;
}

static double draw(int var_kind, double lb, double ub, uint64_t vid,
                   uint64_t i, uint64_t r, uint64_t salt)
{
  return var_kind != CMN_VAR_CONTINUOUS ? orc_sample_discrete(lb, ub, vid, i, r, salt)
                                        : orc_sample_continuous(lb, ub, vid, i, r, salt);
}

/* ======================================================================
 * roles (graph/replay.cuh:610-844)
 * ==================================================================== */
typedef struct {
  const uint8_t* kinds;
  const uint64_t* var_ids;
  const uint64_t* widths;
  int64_t count;
  uint64_t prefix[64];
} slots_t;

static void slots_init(slots_t* s, const uint8_t* kinds, const uint64_t* vids,
                       const uint64_t* widths, int64_t count)
{
  s->kinds = kinds;
  s->var_ids = vids;
  s->widths = widths;
  s->count = count;
  uint64_t running = 1; /* saturating prefix (region/composition.hpp:114-130) */
  for (int64_t j = 0; j < count; ++j) {
    s->prefix[j] = running;
    uint64_t w = widths[j];
    if (w != 0 && running > UINT64_MAX / w) running = UINT64_MAX;
    else running *= w;
  }
}

/* Child box of region r: the parent, narrowed by each slot's digit
 * (graph/kernels.cuh:76-117 broadcast + apply). */
static void child_box(const double* parent, int64_t n, const slots_t* s,
                      uint64_t r, double* out)
{
  memcpy(out, parent, sizeof(double) * 2 * (size_t)n);
  for (int64_t j = 0; j < s->count; ++j) {
    uint64_t part = (r / s->prefix[j]) % s->widths[j];
    uint64_t vid = s->var_ids[j];
    orc_slot_bounds(s->kinds[j], parent[2 * vid], parent[2 * vid + 1], part,
                    s->widths[j], &out[2 * vid], &out[2 * vid + 1]);
  }
}

typedef struct {
  const orc_problem* p;
  const double* box;
  const slots_t* s;
  uint8_t* feas;
  double* obj_lb;
  double* obj_ub; /* optional */
  int failed;
  int hw; /* bound with the hardware directed rounding (_h operators) */
  /* sampling / enumerate */
  uint64_t S, salt;
  int exact;
  double* best_val; /* per thread */
  int64_t* best_idx;
} role_ctx;

static void bound_range(void* vc, int64_t r0, int64_t r1, int tid)
{
  (void)tid;
  role_ctx* c = (role_ctx*)vc;
  const orc_problem* p = c->p;
  double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)p->n_vars);
  iv64* val = (iv64*)malloc(sizeof(iv64) * (size_t)p->n_nodes);
  for (int64_t r = r0; r < r1; ++r) {
    child_box(c->box, p->n_vars, c->s, (uint64_t)r, cb);
    if (c->hw) {
      fesetround(FE_DOWNWARD);
      if (eval_all_hw(p, cb, val)) c->failed = 1;
      fesetround(FE_TONEAREST);
    } else if (eval_all_d(p, cb, val)) {
      c->failed = 1;
    }
    double lb, ub;
    c->feas[r] = (uint8_t)verdict_d(p, val, &lb, &ub);
    c->obj_lb[r] = lb;
    if (c->obj_ub) c->obj_ub[r] = ub;
  }
  free(cb);
  free(val);
}

static int check_widths(const slots_t* s, uint64_t n_regions)
{
  uint64_t total = 1;
  for (int64_t j = 0; j < s->count; ++j) {
    uint64_t w = s->widths[j];
    if (w == 0) return -1;
    if (total > UINT64_MAX / w) return -1;
    total *= w;
  }
  return total == n_regions ? 0 : -1;
}

static int bound_impl(const orc_problem* p, const double* box, const uint8_t* slot_kinds,
                      const uint64_t* var_ids, const uint64_t* widths, int64_t slot_count,
                      uint64_t n_regions, uint8_t* feasible, double* obj_lb, int threads, int hw);

int orc_bound(const orc_problem* p, const double* box,
              const uint8_t* slot_kinds, const uint64_t* var_ids,
              const uint64_t* widths, int64_t slot_count, uint64_t n_regions,
              uint8_t* feasible, double* obj_lb, int threads)
{
  return bound_impl(p, box, slot_kinds, var_ids, widths, slot_count, n_regions, feasible, obj_lb, threads, 0);
}

int orc_bound_hw(const orc_problem* p, const double* box,
                 const uint8_t* slot_kinds, const uint64_t* var_ids,
                 const uint64_t* widths, int64_t slot_count, uint64_t n_regions,
                 uint8_t* feasible, double* obj_lb, int threads)
{
  return bound_impl(p, box, slot_kinds, var_ids, widths, slot_count, n_regions, feasible, obj_lb, threads, 1);
}

static int bound_impl(const orc_problem* p, const double* box, const uint8_t* slot_kinds,
                      const uint64_t* var_ids, const uint64_t* widths, int64_t slot_count,
                      uint64_t n_regions, uint8_t* feasible, double* obj_lb, int threads, int hw)
{
  slots_t s;
  if (slot_count > 64) {
    set_err("slot count above 64");
    return -1;
  }
  slots_init(&s, slot_kinds, var_ids, widths, slot_count);
  if (check_widths(&s, n_regions)) {
    set_err("widths do not multiply out to n_regions");
    return -1;
  }
  role_ctx c;
  memset(&c, 0, sizeof c);
  c.p = p;
  c.box = box;
  c.s = &s;
  c.feas = feasible;
  c.obj_lb = obj_lb;
  c.hw = hw;
  parallel_for((int64_t)n_regions, threads, bound_range, &c);
  if (c.failed) {
    set_err("op without an interval implementation");
    return -1;
  }
  return 0;
}

/* Aggregate bounder (backend/aggregate/kernels.cuh:32-47 mask,
 * backend/aggregate/replay.cuh:343-361 fold, :497-556 reductions):
 * region r belongs to child r / M (M = n_regions / k); a child's lb is the
 * minimum objective lower bound over its feasible regions (+inf when none),
 * its hull_ub the maximum upper bound (-inf when none); a child with
 * hull_ub == -inf is infeasible and normalised to (+inf, +inf).  Minimum and
 * maximum follow the total order of lb_key (-0 below +0, NaN above +inf),
 * which fixes the one choice CUB's Min/Max leave to reduction order. */
static inline uint64_t agg_key(double x)
{
  uint64_t u = dbits(x);
  if (x != x) return UINT64_MAX;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

static inline double agg_unkey(uint64_t k)
{
  uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  return bitsd(u);
}

int orc_aggregate_bound(const orc_problem* p, const double* box,
                        const uint8_t* slot_kinds, const uint64_t* var_ids,
                        const uint64_t* widths, int64_t slot_count,
                        uint64_t n_regions, uint64_t k, double* child_lb,
                        double* child_hull_ub, int32_t* child_feasible,
                        int threads)
{
  if (k == 0 || n_regions % k != 0) {
    set_err("k must divide n_regions");
    return -1;
  }
  slots_t s;
  if (slot_count > 64) {
    set_err("slot count above 64");
    return -1;
  }
  slots_init(&s, slot_kinds, var_ids, widths, slot_count);
  if (check_widths(&s, n_regions)) {
    set_err("widths do not multiply out to n_regions");
    return -1;
  }
  uint8_t* feas = (uint8_t*)malloc(n_regions);
  double* lb = (double*)malloc(sizeof(double) * n_regions);
  double* ub = (double*)malloc(sizeof(double) * n_regions);
  role_ctx c;
  memset(&c, 0, sizeof c);
  c.p = p;
  c.box = box;
  c.s = &s;
  c.feas = feas;
  c.obj_lb = lb;
  c.obj_ub = ub;
  parallel_for((int64_t)n_regions, threads, bound_range, &c);
  int rc = 0;
  if (c.failed) {
    set_err("op without an interval implementation");
    rc = -1;
  }
  const uint64_t M = n_regions / k;
  for (uint64_t ch = 0; ch < k && rc == 0; ++ch) {
    uint64_t kmin = agg_key(INFINITY), kmax = agg_key(-INFINITY);
    for (uint64_t r = ch * M; r < (ch + 1) * M; ++r) {
      const uint64_t a = agg_key(feas[r] ? lb[r] : INFINITY);
      const uint64_t b = agg_key(feas[r] ? ub[r] : -INFINITY);
      if (a < kmin) kmin = a;
      if (b > kmax) kmax = b;
    }
    const double clb = agg_unkey(kmin), cub = agg_unkey(kmax);
    const int f = cub > -INFINITY;
    child_lb[ch] = f ? clb : INFINITY;
    child_hull_ub[ch] = f ? cub : INFINITY;
    child_feasible[ch] = f;
  }
  free(feas);
  free(lb);
  free(ub);
  return rc;
}

/* Sampled point of (region r, sample i): every variable is drawn from its
 * region bound -- the slot's narrowed bound for a slot variable, else the
 * parent bound (subregion_sampler.cuh:133-199: the apply pass overwrites
 * the broadcast pass's draw for slot variables). */
static void sample_point(const orc_problem* p, const double* cb, uint64_t r,
                         uint64_t i, uint64_t salt, double* x)
{
  for (int64_t v = 0; v < p->n_vars; ++v)
    x[v] = draw(p->kinds[v], cb[2 * v], cb[2 * v + 1], (uint64_t)v, i, r, salt);
}

static void sample_range(void* vc, int64_t r0, int64_t r1, int tid)
{
  role_ctx* c = (role_ctx*)vc;
  const orc_problem* p = c->p;
  double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)p->n_vars);
  double* x = (double*)malloc(sizeof(double) * (size_t)p->n_vars);
  double* val = (double*)malloc(sizeof(double) * (size_t)p->n_nodes);
  double best = INFINITY;
  int64_t best_i = -1;
  for (int64_t r = r0; r < r1; ++r) {
    child_box(c->box, p->n_vars, c->s, (uint64_t)r, cb);
    for (uint64_t i = 0; i < c->S; ++i) {
      if (c->exact) {
        for (int64_t v = 0; v < p->n_vars; ++v) x[v] = cb[2 * v];
      } else {
        sample_point(p, cb, (uint64_t)r, i, c->salt, x);
      }
      double obj;
      int f = eval_point_impl(p, x, val, &obj);
      double masked = f ? obj : INFINITY;
      int64_t idx = r * (int64_t)c->S + (int64_t)i;
      if (best_i < 0 || masked < best) { /* first minimal index wins */
        best = masked;
        best_i = idx;
      }
    }
  }
  c->best_val[tid] = best;
  c->best_idx[tid] = best_i;
  free(cb);
  free(x);
  free(val);
}

static int candidate_common(const orc_problem* p, const double* box,
                            const uint8_t* slot_kinds, const uint64_t* var_ids,
                            const uint64_t* widths, int64_t slot_count,
                            uint64_t n_regions, uint64_t S, uint64_t salt,
                            int exact, int32_t* found, double* value,
                            int64_t* index, double* point, int threads)
{
  slots_t s;
  if (slot_count > 64) {
    set_err("slot count above 64");
    return -1;
  }
  slots_init(&s, slot_kinds, var_ids, widths, slot_count);
  if (check_widths(&s, n_regions)) {
    set_err("widths do not multiply out to n_regions");
    return -1;
  }
  if (S < 1) {
    set_err("sample_points must be at least 1");
    return -1;
  }
  role_ctx c;
  memset(&c, 0, sizeof c);
  c.p = p;
  c.box = box;
  c.s = &s;
  c.S = S;
  c.salt = salt;
  c.exact = exact;
  double bv[256];
  int64_t bi[256];
  for (int t = 0; t < 256; ++t) {
    bv[t] = INFINITY;
    bi[t] = -1;
  }
  c.best_val = bv;
  c.best_idx = bi;
  parallel_for((int64_t)n_regions, threads, sample_range, &c);
  /* ArgMin across threads: threads own ascending index ranges, so keeping
   * the first strictly smaller value keeps the first minimal index
   * (graph/replay.cuh:439-474, CUB ArgMin). */
  double best = INFINITY;
  int64_t best_i = -1;
  for (int t = 0; t < 256; ++t) {
    if (bi[t] < 0) continue;
    if (best_i < 0 || bv[t] < best) {
      best = bv[t];
      best_i = bi[t];
    }
  }
  *index = best_i;
  *value = best;
  *found = best < DBL_MAX; /* has_candidate (replay.cuh has_candidate) */
  if (!*found) {
    for (int64_t v = 0; v < p->n_vars; ++v) point[v] = NAN;
    return 0;
  }
  double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)p->n_vars);
  uint64_t r = (uint64_t)best_i / S, i = (uint64_t)best_i % S;
  child_box(box, p->n_vars, &s, r, cb);
  if (exact) {
    for (int64_t v = 0; v < p->n_vars; ++v) point[v] = cb[2 * v];
  } else {
    sample_point(p, cb, r, i, salt, point);
  }
  free(cb);
  return 0;
}

int orc_sample(const orc_problem* p, const double* box,
               const uint8_t* slot_kinds, const uint64_t* var_ids,
               const uint64_t* widths, int64_t slot_count,
               uint64_t n_regions, uint64_t sample_points, uint64_t salt,
               int32_t* found, double* value, int64_t* index, double* point,
               int threads)
{
  return candidate_common(p, box, slot_kinds, var_ids, widths, slot_count,
                          n_regions, sample_points, salt, 0, found, value,
                          index, point, threads);
}

int orc_enumerate(const orc_problem* p, const double* box,
                  const uint8_t* slot_kinds, const uint64_t* var_ids,
                  const uint64_t* widths, int64_t slot_count,
                  uint64_t n_regions, int32_t* found, double* value,
                  int64_t* index, double* point, int threads)
{
  return candidate_common(p, box, slot_kinds, var_ids, widths, slot_count,
                          n_regions, 1, 0, 1, found, value, index, point,
                          threads);
}

/* ======================================================================
 * BisectionBudget policy (policy/bisection_budget.hpp:81-262)
 * ==================================================================== */
typedef struct {
  uint64_t vid;
  int kind;
  uint64_t domain;
  uint64_t bits;
} enum_cand;

typedef struct {
  uint64_t vid;
  int kind;
  double live;
  double orig;
  uint64_t bis;
} bis_cand;

typedef struct {
  const bis_cand* c;
  int relative;
} heap_ctx;

static inline double heap_key(const heap_ctx* h, uint64_t i)
{
  return h->relative ? h->c[i].live / h->c[i].orig : h->c[i].live;
}

static inline int heap_less(const heap_ctx* h, uint64_t a, uint64_t b)
{
  return heap_key(h, a) < heap_key(h, b);
}

/* The policy orders bisection candidates with the C++ standard library's
 * make_heap / pop_heap / push_heap, so which of several equally wide
 * variables is halved first is decided by that heap's layout.  These four
 * functions restate the GCC libstdc++ heap algorithm (hole-based sift-down
 * to a leaf that prefers the right child unless it is smaller than the
 * left, followed by a sift-up) so ties resolve the same way. */
static void hp_push_hole(uint64_t* f, int64_t hole, int64_t top, uint64_t value,
                         const heap_ctx* h)
{
  int64_t parent = (hole - 1) / 2;
  while (hole > top && heap_less(h, f[parent], value)) {
    f[hole] = f[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  f[hole] = value;
}

static void hp_adjust(uint64_t* f, int64_t hole, int64_t len, uint64_t value,
                      const heap_ctx* h)
{
  const int64_t top = hole;
  int64_t second = hole;
  while (second < (len - 1) / 2) {
    second = 2 * (second + 1);
    if (heap_less(h, f[second], f[second - 1])) second--;
    f[hole] = f[second];
    hole = second;
  }
  if ((len & 1) == 0 && second == (len - 2) / 2) {
    second = 2 * (second + 1);
    f[hole] = f[second - 1];
    hole = second - 1;
  }
  hp_push_hole(f, hole, top, value, h);
}

static void hp_make(uint64_t* f, int64_t len, const heap_ctx* h)
{
  if (len < 2) return;
  int64_t parent = (len - 2) / 2;
  for (;;) {
    uint64_t v = f[parent];
    hp_adjust(f, parent, len, v, h);
    if (parent == 0) return;
    parent--;
  }
}

static void hp_pop(uint64_t* f, int64_t len, const heap_ctx* h)
{
  if (len > 1) {
    --len;
    uint64_t v = f[len];
    f[len] = f[0];
    hp_adjust(f, 0, len, v, h);
  }
}

static void hp_push(uint64_t* f, int64_t len, const heap_ctx* h)
{
  uint64_t v = f[len - 1];
  hp_push_hole(f, len - 1, 0, v, h);
}

static uint64_t integer_domain_size(double lb, double ub)
{
  double lo = ceil(lb), hi = floor(ub);
  if (hi < lo) return 0;
  return (uint64_t)(hi - lo) + 1;
}

static uint64_t bits_for(uint64_t d)
{
  uint64_t eff = d == 0 ? 1 : d;
  uint64_t bits = 0, cap = 1;
  while (cap < eff) {
    cap <<= 1;
    ++bits;
  }
  return bits > 1 ? bits : 1;
}

int64_t orc_bisection_choose(const double* box, const int32_t* var_kinds,
                             int64_t n_vars, int64_t B, int64_t max_cycle,
                             int64_t enumerate_cap, int relative,
                             uint8_t* kinds, uint64_t* var_ids,
                             uint64_t* widths, uint64_t* domain_sizes)
{
  int64_t cap = max_cycle == 0 ? 64 : max_cycle;
  enum_cand* ec = (enum_cand*)malloc(sizeof(enum_cand) * (size_t)(n_vars + 1));
  bis_cand* bc = (bis_cand*)malloc(sizeof(bis_cand) * (size_t)(n_vars + 1));
  int64_t ne = 0, nb = 0;
  for (int64_t vid = 0; vid < n_vars && ne + nb < cap; ++vid) {
    double lb = box[2 * vid], ub = box[2 * vid + 1];
    if (!(ub > lb)) continue;
    double w = ub - lb;
    switch (var_kinds[vid]) {
      case CMN_VAR_BINARY:
        ec[ne].vid = (uint64_t)vid;
        ec[ne].kind = CMN_SLOT_BINARY_ENUMERATE;
        ec[ne].domain = 2;
        ec[ne].bits = bits_for(2);
        ++ne;
        break;
      case CMN_VAR_INTEGER: {
        uint64_t d = integer_domain_size(lb, ub);
        uint64_t dm = d > 1 ? d : 1;
        int under = enumerate_cap == 0 || dm <= (uint64_t)enumerate_cap;
        if (under) {
          ec[ne].vid = (uint64_t)vid;
          ec[ne].kind = CMN_SLOT_INTEGER_ENUMERATE;
          ec[ne].domain = d;
          ec[ne].bits = bits_for(d);
          ++ne;
        } else {
          bc[nb].vid = (uint64_t)vid;
          bc[nb].kind = CMN_SLOT_INTEGER_PARTITION;
          bc[nb].live = w;
          bc[nb].orig = w;
          bc[nb].bis = 0;
          ++nb;
        }
        break;
      }
      default:
        bc[nb].vid = (uint64_t)vid;
        bc[nb].kind = CMN_SLOT_CONTINUOUS;
        bc[nb].live = w;
        bc[nb].orig = w;
        bc[nb].bis = 0;
        ++nb;
        break;
    }
  }
  if (ne + nb == 0) {
    free(ec);
    free(bc);
    return 0;
  }
  /* stable sort by bisection cost (std::stable_sort): insertion sort */
  for (int64_t i = 1; i < ne; ++i) {
    enum_cand x = ec[i];
    int64_t j = i - 1;
    while (j >= 0 && x.bits < ec[j].bits) {
      ec[j + 1] = ec[j];
      --j;
    }
    ec[j + 1] = x;
  }
  uint64_t remaining = (uint64_t)B;
  int64_t taken = 0;
  for (; taken < ne; ++taken) {
    if (ec[taken].bits > remaining) break;
    remaining -= ec[taken].bits;
  }
  for (int64_t i = taken; i < ne; ++i) {
    if (ec[i].kind == CMN_SLOT_INTEGER_ENUMERATE) {
      uint64_t vid = ec[i].vid;
      double w = box[2 * vid + 1] - box[2 * vid];
      bc[nb].vid = vid;
      bc[nb].kind = CMN_SLOT_INTEGER_PARTITION;
      bc[nb].live = w;
      bc[nb].orig = w;
      bc[nb].bis = 0;
      ++nb;
    }
  }
  uint64_t* heap = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(nb + 1));
  for (int64_t i = 0; i < nb; ++i) heap[i] = (uint64_t)i;
  heap_ctx h = {bc, relative};
  hp_make(heap, nb, &h);
  uint64_t spent = 0;
  for (; spent < remaining && nb > 0; ++spent) {
    hp_pop(heap, nb, &h);
    bis_cand* c = &bc[heap[nb - 1]];
    c->live = c->live / 2.0;
    ++c->bis;
    hp_push(heap, nb, &h);
  }
  if (spent < remaining) {
    for (uint64_t k = spent; k < remaining; ++k) {
      int64_t widest = 0;
      for (int64_t i = 1; i < taken; ++i)
        if (ec[i].bits > ec[widest].bits) widest = i;
      ++ec[widest].bits;
    }
  }
  int64_t out = 0;
  for (int64_t i = 0; i < taken; ++i) {
    kinds[out] = (uint8_t)ec[i].kind;
    var_ids[out] = ec[i].vid;
    widths[out] = (uint64_t)1 << ec[i].bits;
    domain_sizes[out] = ec[i].domain;
    ++out;
  }
  for (int64_t i = 0; i < nb; ++i) {
    if (bc[i].bis == 0) continue;
    kinds[out] = (uint8_t)bc[i].kind;
    var_ids[out] = bc[i].vid;
    uint64_t w = (uint64_t)1 << bc[i].bis;
    widths[out] = w;
    domain_sizes[out] = w;
    ++out;
  }
  free(heap);
  free(ec);
  free(bc);
  return out;
}

/* ======================================================================
 * shared search helpers (search/budget.hpp, search/epilogue.hpp)
 * ==================================================================== */
static int gap_closed(double gub, double bound, double tol)
{
  return gub - bound <= tol * fmax(1.0, fabs(gub));
}

static int witness_is_admissible(const orc_problem* p, const double* x)
{
  for (int64_t i = 0; i < p->n_vars; ++i) {
    double v = x[i];
    if (!(v >= p->var_lb[i]) || !(v <= p->var_ub[i])) return 0;
    if (p->kinds[i] == CMN_VAR_INTEGER || p->kinds[i] == CMN_VAR_BINARY) {
      double nearest = round(v);
      if (fabs(v - nearest) > 1e-6) return 0;
    }
  }
  return 1;
}

typedef struct {
  double lb_min;
  uint64_t viable, dominated;
} drop_acc;

static void drop_fold(drop_acc* d, double lb, double gub)
{
  if (lb <= gub) {
    d->lb_min = fmin(d->lb_min, lb);
    ++d->viable;
  } else {
    ++d->dominated;
  }
}

static void finalise(double glb, double gub, double tol, int found,
                     int converged, int pending_empty, double frontier_min,
                     uint64_t viable, const drop_acc* d, cmn_outcome* out)
{
  out->proven_optimal = found && (converged || pending_empty || viable == 0) &&
                        gap_closed(gub, d->lb_min, tol);
  out->infeasible = 0;
  if (out->proven_optimal) {
    out->lower_bound = gub;
  } else if (pending_empty && d->viable == 0) {
    out->infeasible = 1;
    out->lower_bound = glb;
  } else {
    double frontier = pending_empty ? DBL_MAX : frontier_min;
    double g = fmin(frontier, d->lb_min);
    if (found) g = fmin(g, gub);
    out->lower_bound = g;
  }
}

int orc_finalise(double glb, double gub, double tol, int found, int converged, int pending_empty,
                 double frontier_min, uint64_t viable, const double* drop_lbs, const double* drop_gubs,
                 int64_t n_drops, cmn_outcome* out)
{
  drop_acc d = {INFINITY, 0, 0};
  for (int64_t i = 0; i < n_drops; ++i) drop_fold(&d, drop_lbs[i], drop_gubs[i]);
  finalise(glb, gub, tol, found, converged, pending_empty, frontier_min, viable, &d, out);
  return 0;
}

static uint64_t slot_product(const uint64_t* widths, int64_t count)
{
  uint64_t total = 1;
  for (int64_t j = 0; j < count; ++j) {
    uint64_t w = widths[j];
    if (w != 0 && total > UINT64_MAX / w) return UINT64_MAX;
    total *= w;
  }
  return total;
}

static int fully_enumerable(const uint8_t* kinds, int64_t count)
{
  for (int64_t j = 0; j < count; ++j)
    if (kinds[j] != CMN_SLOT_INTEGER_ENUMERATE && kinds[j] != CMN_SLOT_BINARY_ENUMERATE)
      return 0;
  return 1;
}

static int is_dup(uint64_t r, const slots_t* s, const uint64_t* domain)
{
  for (int64_t j = 0; j < s->count; ++j) {
    uint64_t part = (r / s->prefix[j]) % s->widths[j];
    if (part >= domain[j]) return 1;
  }
  return 0;
}

static void opts_norm(const cmn_solve_options* o, cmn_solve_options* n)
{
  *n = *o;
  if (n->sample_points == 0) n->sample_points = 1;
  if (n->batch_parents == 0) n->batch_parents = 1;
  if (n->bisection_budget < 1) n->bisection_budget = 1;
}

/* ======================================================================
 * reference driver restatement (search/driver.hpp:137-537 with
 * search/frontier.hpp:44-338 Node order and IntervalPQueue heap,
 * search/history.hpp:20-137 refcounted history)
 * ==================================================================== */
typedef struct {
  uint64_t sidx, pidx, depth;
  double lb;
} rnode;

static int rnode_less(const rnode* a, const rnode* b)
{
  if (a->lb < b->lb) return 1;
  if (b->lb < a->lb) return 0;
  if (a->depth != b->depth) return a->depth > b->depth;
  return a->pidx > b->pidx;
}

typedef struct {
  rnode* e;
  uint64_t n, cap;
} rheap;

static void rh_push(rheap* h, rnode x)
{
  if (h->n == h->cap) {
    h->cap = h->cap ? h->cap * 2 : 1024;
    h->e = (rnode*)realloc(h->e, sizeof(rnode) * h->cap);
  }
  uint64_t idx = h->n++;
  while (idx != 0 && rnode_less(&x, &h->e[(idx - 1) / 2])) {
    h->e[idx] = h->e[(idx - 1) / 2];
    idx = (idx - 1) / 2;
  }
  h->e[idx] = x;
}

static rnode rh_pop(rheap* h)
{
  rnode res = h->e[0];
  --h->n;
  if (h->n > 0) {
    rnode x = h->e[h->n];
    uint64_t idx = 0;
    while (2 * idx + 1 < h->n) {
      uint64_t l = 2 * idx + 1, r = 2 * idx + 2;
      uint64_t child = (r < h->n && rnode_less(&h->e[r], &h->e[l])) ? r : l;
      if (!rnode_less(&h->e[child], &x)) break;
      h->e[idx] = h->e[child];
      idx = child;
    }
    h->e[idx] = x;
  }
  return res;
}

typedef struct {
  double* box; /* 2n */
  uint8_t kinds[64];
  uint64_t vids[64], widths[64];
  int64_t count;
  uint64_t refs;
} hist_entry;

typedef struct {
  hist_entry* e;
  uint64_t n, cap;
  uint64_t* free_slots;
  uint64_t n_free, free_cap;
} history;

static uint64_t hist_enqueue(history* h, const double* box, int64_t nvars)
{
  uint64_t idx;
  if (h->n_free > 0) {
    idx = h->free_slots[--h->n_free];
  } else {
    if (h->n == h->cap) {
      h->cap = h->cap ? h->cap * 2 : 256;
      h->e = (hist_entry*)realloc(h->e, sizeof(hist_entry) * h->cap);
    }
    idx = h->n++;
    h->e[idx].box = NULL;
  }
  hist_entry* e = &h->e[idx];
  if (!e->box) e->box = (double*)malloc(sizeof(double) * 2 * (size_t)(nvars > 0 ? nvars : 1));
  if (box) memcpy(e->box, box, sizeof(double) * 2 * (size_t)nvars);
  e->refs = 1;
  e->count = 0;
  return idx;
}

static void hist_add_ref(history* h, uint64_t idx)
{
  if (idx == 0) return;
  ++h->e[idx].refs;
}

static void hist_release(history* h, uint64_t idx)
{
  if (idx == 0) return;
  if (--h->e[idx].refs > 0) return;
  if (h->n_free == h->free_cap) {
    h->free_cap = h->free_cap ? h->free_cap * 2 : 256;
    h->free_slots = (uint64_t*)realloc(h->free_slots, sizeof(uint64_t) * h->free_cap);
  }
  h->free_slots[h->n_free++] = idx;
}

int orc_solve_reference(const orc_problem* p, const cmn_solve_options* opts_in,
                        cmn_outcome* out, double* best_point, int threads)
{
  cmn_solve_options o;
  opts_norm(opts_in, &o);
  const int64_t n = p->n_vars;
  memset(out, 0, sizeof *out);
  double GUB = o.has_known_primal ? o.known_primal_bound : DBL_MAX;
  double GLB = -DBL_MAX;
  uint64_t iter = 0;
  int have_best = 0;
  rheap pending = {0, 0, 0};
  history hist;
  memset(&hist, 0, sizeof hist);
  hist_enqueue(&hist, NULL, n); /* root sentinel */
  rnode root = {0, 0, 0, GLB};
  rh_push(&pending, root);

  cmn_counters* ct = &out->counters;
  drop_acc dropped = {INFINITY, 0, 0};
  int converged = 0, stopped_early = 0, stop = CMN_STOP_ITERATION_LIMIT;
  uint64_t N = (uint64_t)1 << o.bisection_budget;
  double* box = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  uint8_t* feas = (uint8_t*)malloc(N);
  double* olb = (double*)malloc(sizeof(double) * N);
  double* pt = (double*)malloc(sizeof(double) * (size_t)n);
  uint8_t kinds[64];
  uint64_t vids[64], widths[64], dom[64];
  int rc = 0;

  while (iter < o.iter_limit && pending.n > 0 && !gap_closed(GUB, GLB, o.tolerance)) {
    ++iter;
    rnode cur = rh_pop(&pending);
    if (gap_closed(GUB, cur.lb, o.tolerance)) {
      converged = 1;
      stop = CMN_STOP_CONVERGED;
      stopped_early = 1;
      break;
    }
    GLB = cur.lb;
    /* materialise (search/frontier.hpp:113-144) */
    if (cur.pidx == 0) {
      for (int64_t v = 0; v < n; ++v) {
        box[2 * v] = p->var_lb[v];
        box[2 * v + 1] = p->var_ub[v];
      }
    } else {
      hist_entry* pe = &hist.e[cur.pidx];
      slots_t ps;
      slots_init(&ps, pe->kinds, pe->vids, pe->widths, pe->count);
      child_box(pe->box, n, &ps, cur.sidx, box);
    }
    hist_release(&hist, cur.pidx);

    int64_t sc = orc_bisection_choose(box, p->kinds, n, o.bisection_budget,
                                      (int64_t)o.max_cycle_size, (int64_t)o.enumerate_cap,
                                      o.relative_width, kinds, vids, widths, dom);
    int64_t live = 0;
    for (int64_t v = 0; v < n; ++v)
      if (box[2 * v + 1] > box[2 * v]) ++live;
    uint64_t nreg = sc == 0 ? 1 : slot_product(widths, sc);

    if (live <= sc && fully_enumerable(kinds, sc)) {
      int32_t found;
      double value;
      int64_t index;
      if (orc_enumerate(p, box, kinds, vids, widths, sc, nreg, &found, &value, &index, pt, threads)) {
        rc = -1;
        break;
      }
      if (found && value < GUB) {
        if (witness_is_admissible(p, pt)) {
          GUB = value;
          memcpy(best_point, pt, sizeof(double) * (size_t)n);
          have_best = 1;
        } else {
          ++ct->witness_rejected;
        }
      }
      ++ct->fathomed;
      ct->fathomed_points += nreg;
      continue;
    }

    uint64_t box_idx = hist_enqueue(&hist, box, n);
    {
      hist_entry* he = &hist.e[box_idx];
      he->count = sc;
      memcpy(he->kinds, kinds, (size_t)sc);
      memcpy(he->vids, vids, sizeof(uint64_t) * (size_t)sc);
      memcpy(he->widths, widths, sizeof(uint64_t) * (size_t)sc);
    }
    int32_t found;
    double value;
    int64_t index;
    if (orc_sample(p, box, kinds, vids, widths, sc, nreg, o.sample_points, iter, &found,
                   &value, &index, pt, threads)) {
      rc = -1;
      break;
    }
    ct->sampled += nreg * o.sample_points;
    if (value < GUB) {
      if (witness_is_admissible(p, pt)) {
        GUB = value;
        memcpy(best_point, pt, sizeof(double) * (size_t)n);
        have_best = 1;
      } else {
        ++ct->witness_rejected;
      }
    }
    if (orc_bound(p, box, kinds, vids, widths, sc, nreg, feas, olb, threads)) {
      rc = -1;
      break;
    }
    ct->bounded += nreg;
    slots_t s;
    slots_init(&s, kinds, vids, widths, sc);
    for (uint64_t t = 0; t < nreg; ++t) {
      if (is_dup(t, &s, dom)) {
        ++ct->pruned_duplicate;
        continue;
      }
      if (!feas[t]) {
        ++ct->pruned_infeasible;
        continue;
      }
      if (olb[t] > GUB) {
        ++ct->pruned_dominated;
        continue;
      }
      rnode c = {t, box_idx, cur.depth + 1, olb[t]};
      rh_push(&pending, c);
      hist_add_ref(&hist, box_idx);
      ++ct->enqueued;
    }
    hist_release(&hist, box_idx);
    if (pending.n > ct->peak_frontier) ct->peak_frontier = pending.n;
  }

  if (!stopped_early)
    stop = pending.n == 0 ? CMN_STOP_EXHAUSTED
           : gap_closed(GUB, GLB, o.tolerance) ? CMN_STOP_CONVERGED
                                               : CMN_STOP_ITERATION_LIMIT;
  int found = GUB < DBL_MAX;
  uint64_t viable = 0;
  double fmin_lb = DBL_MAX;
  for (uint64_t i = 0; i < pending.n; ++i) {
    if (pending.e[i].lb <= GUB) ++viable;
  }
  if (pending.n > 0) fmin_lb = pending.e[0].lb;
  finalise(GLB, GUB, o.tolerance, found, converged, pending.n == 0, fmin_lb, viable, &dropped, out);
  out->upper_bound = GUB;
  out->stop_reason = stop;
  out->found_incumbent = found;
  out->frontier_size = pending.n;
  out->viable = viable;
  out->dropped_lb_min = dropped.lb_min;
  ct->iterations = iter;
  ct->expansions = iter;
  if (!have_best)
    for (int64_t v = 0; v < n; ++v) best_point[v] = NAN;
  for (uint64_t i = 0; i < hist.n; ++i) free(hist.e[i].box);
  free(hist.e);
  free(hist.free_slots);
  free(pending.e);
  free(box);
  free(feas);
  free(olb);
  free(pt);
  return rc;
}

/* ======================================================================
 * the lazy form's incremental FP32 children, restated from the device
 * (csrc/eval_kernels.cu inc_common_kernel / eval_children_inc_kernel)
 * over the library's compiled FP32 program (cmn_problem_program)
 * ==================================================================== */
/* One instruction of the compiled program, 16 bytes (cmn_problem_program). */
struct orc_instr {
  uint8_t head, modes;
  uint16_t dst, a, b;
  union {
    double c;
    struct {
      float clo, chi;
    } c32;
  } u;
};

enum { OP_GENERIC = 0, OP_TERM = 1, OP_STOREACC = 2, OP_LOADACC = 3, OP_CONSTTOSLOT = 4, OP_CHECK = 5,
       OP_OBJECTIVE = 6 };
enum { MODE_SLOT = 0, MODE_VAR = 1, MODE_ACC = 2, MODE_CONST = 3 };
enum { T_INIT = 1, T_SUB = 2, T_HASC = 4, T_SQR = 8, T_VAR = 16, T_PMASK = 24 };

/* Segments and per-(variable, segment) chain lists, derived here from the
 * instruction stream independently of the library's own tables: a
 * segment is a sum chain (a LoadAcc or an initialising TERM, then TERMs)
 * followed by the checks and objective that read it. */
int orc_set_program64(orc_problem* p, const void* instrs, int64_t len)
{
  free(p->prog64);
  p->prog64 = NULL;
  p->prog64_len = 0;
  p->n_prog_slots = 0;
  if (len <= 0) return 0;
  p->prog64 = (struct orc_instr*)malloc(sizeof(struct orc_instr) * (size_t)len);
  memcpy(p->prog64, instrs, sizeof(struct orc_instr) * (size_t)len);
  p->prog64_len = len;
  for (int64_t pc = 0; pc < len; ++pc) {
    const struct orc_instr* in = &p->prog64[pc];
    const int op = in->head & 7;
    if (op == OP_GENERIC || op == OP_STOREACC || op == OP_CONSTTOSLOT)
      if ((int64_t)in->dst + 1 > p->n_prog_slots) p->n_prog_slots = (int64_t)in->dst + 1;
  }
  return 1;
}

static iv64 prog_fetch64(const struct orc_instr* in, int mode, int idx, const double* box, const iv64* slots,
                         iv64 acc)
{
  iv64 v;
  switch (mode) {
    case MODE_SLOT: return slots[idx];
    case MODE_VAR:
      v.lo = box[2 * idx];
      v.hi = box[2 * idx + 1];
      return v;
    case MODE_ACC: return acc;
    default:
      v.lo = in->u.c;
      v.hi = in->u.c;
      return v;
  }
}

/* Box `box` (lo, hi pairs) through the FP64 program (orc_set_program64),
 * restating csrc/eval_core.cuh interval_range.  With `fused` set, the lazy
 * form's verdict: a TERM with a coefficient c that adds into its chain
 * folds c and the add into one directed FMA per bound (the coefficient's
 * sign picks the product's endpoint).  Without it, and for every other
 * instruction, the program's operations each round on their own, as the
 * plain form runs them.  Runs under FE_DOWNWARD with the _h operators
 * (round-up as negated round-down, fma included).  Returns the reference
 * predicate (1 feasible), or -1 for an operator without an interval form;
 * *lb, *ub the objective's enclosure.  `slots` has room for the program's
 * slots. */
static int program_run64(const orc_problem* p, const double* box, iv64* slots, double* lb, double* ub, int fused)
{
  iv64 acc = {0.0, 0.0};
  iv64 obj = {NAN, NAN};
  int feas = 1, rc = 0;
  fesetround(FE_DOWNWARD);
  for (int64_t pc = 0; pc < p->prog64_len && rc == 0; ++pc) {
    const struct orc_instr* in = &p->prog64[pc];
    const int op = in->head & 7, sub = in->head >> 3;
    switch (op) {
      case OP_TERM: {
        iv64 xa = prog_fetch64(in, MODE_VAR, in->a, box, slots, acc);
        iv64 xb = prog_fetch64(in, MODE_VAR, in->b, box, slots, acc);
        const int pk = sub & T_PMASK;
        iv64 prod = pk == T_SQR ? iv_sqr_h(xa) : (pk == T_VAR ? xa : iv_mul_h(xa, xb));
        if (fused && (sub & T_HASC) && !(sub & T_INIT)) {
          const double cc = (sub & T_SUB) ? -in->u.c : in->u.c;
          const int pos = cc >= 0.0;
          acc.lo = fma(cc, pos ? prod.lo : prod.hi, acc.lo);
          acc.hi = -fma(-cc, pos ? prod.hi : prod.lo, -acc.hi);
        } else {
          iv64 t = prod;
          if (sub & T_HASC) {
            iv64 c = {in->u.c, in->u.c};
            t = iv_mul_h(c, prod);
          }
          acc = (sub & T_INIT) ? t : ((sub & T_SUB) ? iv_sub_h(acc, t) : iv_add_h(acc, t));
        }
        break;
      }
      case OP_GENERIC: {
        if (!op_supported_interval(sub)) {
          rc = -1;
          break;
        }
        iv64 a = prog_fetch64(in, in->modes & 3, in->a, box, slots, acc);
        iv64 b = prog_fetch64(in, (in->modes >> 2) & 3, in->b, box, slots, acc);
        slots[in->dst] = apply_hw(sub, a, b, (int)(int16_t)in->b);
        break;
      }
      case OP_STOREACC: slots[in->dst] = acc; break;
      case OP_LOADACC: acc = prog_fetch64(in, in->modes & 3, in->a, box, slots, acc); break;
      case OP_CONSTTOSLOT:
        slots[in->dst].lo = in->u.c;
        slots[in->dst].hi = in->u.c;
        break;
      case OP_CHECK: {
        iv64 v = prog_fetch64(in, in->modes & 3, in->a, box, slots, acc);
        const double rhs = in->u.c;
        if (sub == 0) feas = feas && (v.lo <= rhs);
        else feas = feas && (v.lo <= rhs && rhs <= v.hi);
        break;
      }
      case OP_OBJECTIVE: obj = prog_fetch64(in, in->modes & 3, in->a, box, slots, acc); break;
      default: break;
    }
  }
  fesetround(FE_TONEAREST);
  *lb = obj.lo;
  *ub = obj.hi;
  return rc ? rc : feas;
}

int orc_program_eval64(const orc_problem* p, const double* box, double* lb, double* ub)
{
  if (!p->prog64) {
    set_err("no FP64 program: call orc_set_program64 first");
    return -2;
  }
  iv64* slots = (iv64*)malloc(sizeof(iv64) * (size_t)(p->n_prog_slots > 0 ? p->n_prog_slots : 1));
  const int f = program_run64(p, box, slots, lb, ub, 0);
  free(slots);
  if (f < 0) set_err("op without an interval implementation");
  return f;
}

/* An FP32 program operand: variables widened outward on conversion,
 * constants as the program's outward-rounded pair (csrc/eval_core.cuh
 * const_of<float>). */
static iv32 prog_fetch32(const struct orc_instr* in, int mode, int idx, const double* box, const iv32* slots,
                         iv32 acc)
{
  iv32 v;
  switch (mode) {
    case MODE_SLOT: return slots[idx];
    case MODE_VAR:
      v.lo = orc_d2f_rd(box[2 * idx]);
      v.hi = orc_d2f_ru(box[2 * idx + 1]);
      return v;
    case MODE_ACC: return acc;
    default:
      v.lo = in->u.c32.clo;
      v.hi = in->u.c32.chi;
      return v;
  }
}

int orc_program_eval32(const orc_problem* p, const double* box, double* lb, double* ub)
{
  if (!p->prog32) {
    set_err("no FP32 program: call orc_set_program32 first");
    return -2;
  }
  int64_t n_slots = 1;
  for (int64_t pc = 0; pc < p->prog_len; ++pc) {
    const int op = p->prog32[pc].head & 7;
    if (op == OP_GENERIC || op == OP_STOREACC || op == OP_CONSTTOSLOT)
      if ((int64_t)p->prog32[pc].dst + 1 > n_slots) n_slots = (int64_t)p->prog32[pc].dst + 1;
  }
  iv32* slots = (iv32*)malloc(sizeof(iv32) * (size_t)n_slots);
  iv32 acc = {0.0f, 0.0f};
  iv32 obj = {NAN, NAN};
  int excluded = 0, rc = 0;
  for (int64_t pc = 0; pc < p->prog_len && rc == 0; ++pc) {
    const struct orc_instr* in = &p->prog32[pc];
    const int op = in->head & 7, sub = in->head >> 3;
    switch (op) {
      case OP_TERM: {
        const iv32 xa = prog_fetch32(in, MODE_VAR, in->a, box, slots, acc);
        const iv32 xb = prog_fetch32(in, MODE_VAR, in->b, box, slots, acc);
        const int pk = sub & T_PMASK;
        iv32 t = pk == T_SQR ? iv_sqr_f(xa) : (pk == T_VAR ? xa : iv_mul_f(xa, xb));
        if (sub & T_HASC) {
          const iv32 c = {in->u.c32.clo, in->u.c32.chi};
          t = iv_mul_f(c, t);
        }
        acc = (sub & T_INIT) ? t : ((sub & T_SUB) ? iv_sub_f(acc, t) : iv_add_f(acc, t));
        break;
      }
      case OP_GENERIC: {
        if (!op_supported_interval(sub)) {
          rc = -1;
          break;
        }
        const iv32 a = prog_fetch32(in, in->modes & 3, in->a, box, slots, acc);
        const iv32 b = prog_fetch32(in, (in->modes >> 2) & 3, in->b, box, slots, acc);
        slots[in->dst] = apply_f(sub, a, b, (int)(int16_t)in->b);
        break;
      }
      case OP_STOREACC: slots[in->dst] = acc; break;
      case OP_LOADACC: acc = prog_fetch32(in, in->modes & 3, in->a, box, slots, acc); break;
      case OP_CONSTTOSLOT:
        slots[in->dst].lo = in->u.c32.clo;
        slots[in->dst].hi = in->u.c32.chi;
        break;
      case OP_CHECK: { /* the rhs stays FP64 in both programs; "proven violated" */
        const iv32 v = prog_fetch32(in, in->modes & 3, in->a, box, slots, acc);
        const double rhs = in->u.c;
        if (sub == 0) excluded = excluded || ((double)v.lo > rhs);
        else excluded = excluded || ((double)v.lo > rhs || (double)v.hi < rhs);
        break;
      }
      case OP_OBJECTIVE: obj = prog_fetch32(in, in->modes & 3, in->a, box, slots, acc); break;
      default: break;
    }
  }
  free(slots);
  *lb = (double)obj.lo;
  *ub = (double)obj.hi;
  if (rc < 0) set_err("op without an interval implementation");
  return rc < 0 ? rc : !excluded;
}

int orc_set_program32(orc_problem* p, const void* instrs, int64_t len)
{
  free(p->prog32);
  free(p->inc_seg);
  free(p->inc_off);
  free(p->inc_pcs);
  p->prog32 = NULL;
  p->inc_seg = p->inc_off = p->inc_pcs = NULL;
  p->inc_ok = 0;
  p->prog_len = len;
  if (len <= 0) return 0;
  p->prog32 = (struct orc_instr*)malloc(sizeof(struct orc_instr) * (size_t)len);
  memcpy(p->prog32, instrs, sizeof(struct orc_instr) * (size_t)len);
  const struct orc_instr* code = p->prog32;
  int32_t* seg = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)(len + 1));
  int64_t S = 0, pc = 0;
#define ACCUM(in) (((in).head & 7) == OP_TERM || ((in).head & 7) == OP_LOADACC)
#define STARTS(in) ((((in).head & 7) == OP_TERM && (((in).head >> 3) & T_INIT)) || ((in).head & 7) == OP_LOADACC)
  while (pc < len) {
    int64_t b = pc, t = pc, e;
    if (STARTS(code[pc])) {
      t = pc + 1;
      while (t < len && ACCUM(code[t]) && !STARTS(code[t])) ++t;
    }
    e = t;
    while (e < len && !ACCUM(code[e])) {
      int c = code[e].head & 7;
      if (c != OP_CHECK && c != OP_OBJECTIVE) {
        free(seg);
        return 0;
      }
      ++e;
    }
    if (e == b) {
      free(seg);
      return 0;
    }
    seg[3 * S] = (int32_t)b;
    seg[3 * S + 1] = (int32_t)t;
    seg[3 * S + 2] = (int32_t)e;
    ++S;
    pc = e;
  }
#undef ACCUM
#undef STARTS
  const int64_t n = p->n_vars;
  int32_t* cnt = (int32_t*)calloc((size_t)(n * S + 1), sizeof(int32_t));
  for (int pass = 0; pass < 2; ++pass) {
    int32_t* fill = pass ? (int32_t*)calloc((size_t)(n * S + 1), sizeof(int32_t)) : NULL;
    for (int64_t s = 0; s < S; ++s) {
      for (int32_t q = seg[3 * s]; q < seg[3 * s + 1]; ++q) {
        const struct orc_instr* in = &code[q];
        int va = -1, vb = -1;
        if ((in->head & 7) == OP_TERM) {
          va = in->a;
          vb = in->b;
        } else if ((in->modes & 3) == MODE_VAR) {
          va = vb = in->a;
        }
        int vs[2] = {va, vb != va ? vb : -1};
        for (int w = 0; w < 2; ++w) {
          if (vs[w] < 0) continue;
          if (vs[w] >= n) {
            free(seg);
            free(cnt);
            free(fill);
            return 0;
          }
          int64_t slot = vs[w] * S + s;
          if (!pass) ++cnt[slot];
          else p->inc_pcs[p->inc_off[slot] + fill[slot]++] = q;
        }
      }
    }
    if (!pass) {
      p->inc_off = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * S + 1));
      int32_t acc = 0;
      for (int64_t i = 0; i < n * S; ++i) {
        p->inc_off[i] = acc;
        acc += cnt[i];
      }
      p->inc_off[n * S] = acc;
      p->inc_pcs = (int32_t*)malloc(sizeof(int32_t) * (size_t)(acc ? acc : 1));
    } else {
      free(fill);
    }
  }
  free(cnt);
  p->inc_seg = seg;
  p->inc_segments = S;
  p->inc_ok = 1;
  return 1;
}

/* x of a box as an FP32 interval: box holds FP32 (lo, hi) per variable */
static iv32 term_value_f(const struct orc_instr* in, const iv32* x)
{
  const int sub = in->head >> 3, pk = sub & T_PMASK;
  iv32 r;
  if (pk == 0) r = iv_mul_f(x[in->a], x[in->b]);
  else if (pk == T_SQR) r = iv_sqr_f(x[in->a]);
  else r = x[in->a];
  if (sub & T_HASC) {
    iv32 c = {in->u.c32.clo, in->u.c32.chi};
    r = iv_mul_f(c, r);
  }
  return r;
}

static iv32 chain_add_f(iv32 acc, const struct orc_instr* in, const iv32* x)
{
  if ((in->head & 7) == OP_TERM) {
    iv32 t = term_value_f(in, x);
    return ((in->head >> 3) & T_SUB) ? iv_sub_f(acc, t) : iv_add_f(acc, t);
  }
  iv32 v;
  if ((in->modes & 3) == MODE_VAR) {
    v = x[in->a];
  } else {
    v.lo = in->u.c32.clo;
    v.hi = in->u.c32.chi;
  }
  return iv_add_f(acc, v);
}

/* the FP32 box of parent box `pb` (FP64 lo/hi pairs) rounded outward */
static void box32(const orc_problem* p, const double* pb, iv32* x)
{
  for (int64_t v = 0; v < p->n_vars; ++v) {
    x[v].lo = orc_d2f_rd(pb[2 * v]);
    x[v].hi = orc_d2f_ru(pb[2 * v + 1]);
  }
}

/* common chain sums of one parent (its split variables `vids[0..count)`):
 * out[2s], out[2s+1] */
static void inc_common_one(const orc_problem* p, const double* pb, const uint64_t* vids, int64_t count,
                           iv32* x, float* out)
{
  box32(p, pb, x);
  for (int64_t s = 0; s < p->inc_segments; ++s) {
    iv32 acc = {0.0f, 0.0f};
    for (int32_t q = p->inc_seg[3 * s]; q < p->inc_seg[3 * s + 1]; ++q) {
      const struct orc_instr* in = &p->prog32[q];
      const int term = (in->head & 7) == OP_TERM;
      int skip = 0;
      if (term || (in->modes & 3) == MODE_VAR) {
        for (int64_t j = 0; j < count; ++j)
          if (vids[j] == in->a || (term && vids[j] == in->b)) skip = 1;
      }
      if (!skip) acc = chain_add_f(acc, in, x);
    }
    out[2 * s] = acc.lo;
    out[2 * s + 1] = acc.hi;
  }
}

static int split_before_o(const uint64_t* vids, int64_t j, uint64_t v)
{
  for (int64_t q = 0; q < j; ++q)
    if (vids[q] == v) return 1;
  return 0;
}

/* the child box `cb` (FP64) of parent box `pb` with the given common sums
 * and split variables: FP32 verdict (1 unless a constraint is proven
 * violated), lb, ub.  Per segment: the common sum, then in slot order the
 * part sum of each slot j -- from zero, in program order, the segment's
 * terms reading slot j's variable and no variable of an earlier slot, with
 * that variable over the child's part and every other variable over the
 * parent's bounds (a variable an earlier slot already splits adds
 * nothing) -- then the checks and the objective
 * (csrc/eval_kernels.cu inc_parts_kernel, eval_children_inc_kernel).
 * `x` and `xs` have room for n_vars intervals each. */
static int inc_child(const orc_problem* p, const double* pb, const double* cb, const float* common,
                     const uint64_t* vids, int64_t count, iv32* x, iv32* xs, double* lb, double* ub)
{
  box32(p, cb, x);
  const int64_t S = p->inc_segments;
  /* part sums per (slot, segment) */
  iv32* part = (iv32*)malloc(sizeof(iv32) * (size_t)(count * S > 0 ? count * S : 1));
  for (int64_t j = 0; j < count; ++j) {
    const uint64_t vj = vids[j];
    const int repeated = split_before_o(vids, j, vj);
    box32(p, pb, xs);
    xs[vj] = x[vj];
    for (int64_t s = 0; s < S; ++s) {
      iv32 acc = {0.0f, 0.0f};
      if (!repeated) {
        for (int32_t q = p->inc_off[vj * S + s]; q < p->inc_off[vj * S + s + 1]; ++q) {
          const struct orc_instr* in = &p->prog32[p->inc_pcs[q]];
          if ((in->head & 7) == OP_TERM) {
            uint64_t other = in->a == vj ? in->b : in->a;
            if (other != vj && split_before_o(vids, j, other)) continue;
          }
          acc = chain_add_f(acc, in, xs);
        }
      }
      part[j * S + s] = acc;
    }
  }
  int feas = 1;
  iv32 obj = {NAN, NAN};
  for (int64_t s = 0; s < S; ++s) {
    iv32 acc = {common[2 * s], common[2 * s + 1]};
    for (int64_t j = 0; j < count; ++j) acc = iv_add_f(acc, part[j * S + s]);
    for (int32_t q = p->inc_seg[3 * s + 1]; q < p->inc_seg[3 * s + 2]; ++q) {
      const struct orc_instr* in = &p->prog32[q];
      const int mode = in->modes & 3;
      iv32 v;
      if (mode == MODE_ACC) v = acc;
      else if (mode == MODE_VAR) v = x[in->a];
      else {
        v.lo = in->u.c32.clo;
        v.hi = in->u.c32.chi;
      }
      if ((in->head & 7) == OP_CHECK) {
        double rhs = in->u.c;
        int excluded = ((in->head >> 3) == 0) ? ((double)v.lo > rhs) : ((double)v.lo > rhs || (double)v.hi < rhs);
        if (excluded) feas = 0;
      } else if ((in->head & 7) == OP_OBJECTIVE) {
        obj = v;
      }
    }
  }
  free(part);
  *lb = (double)obj.lo;
  *ub = (double)obj.hi;
  return feas;
}

/* The lazy form's incremental FP32 bound of every region of one parent
 * box (the slot plan as orc_bound takes it): feasible[r] is 0 when the
 * FP32 enclosure proves a constraint violated.  For soundness tests
 * against the FP64 bound. */
int orc_bound_inc32(const orc_problem* p, const double* box, const uint8_t* slot_kinds, const uint64_t* var_ids,
                    const uint64_t* widths, int64_t slot_count, uint64_t n_regions, uint8_t* feasible,
                    double* obj_lb, double* obj_ub)
{
  if (!p->inc_ok) {
    set_err("no incremental program set (orc_set_program32)");
    return -1;
  }
  slots_t s;
  if (slot_count > 64) {
    set_err("slot count above 64");
    return -1;
  }
  slots_init(&s, slot_kinds, var_ids, widths, slot_count);
  if (check_widths(&s, n_regions)) {
    set_err("widths do not multiply out to n_regions");
    return -1;
  }
  const int64_t n = p->n_vars;
  iv32* x = (iv32*)malloc(sizeof(iv32) * (size_t)(n ? n : 1));
  iv32* xs = (iv32*)malloc(sizeof(iv32) * (size_t)(n ? n : 1));
  float* common = (float*)malloc(sizeof(float) * 2 * (size_t)(p->inc_segments ? p->inc_segments : 1));
  double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)(n ? n : 1));
  inc_common_one(p, box, var_ids, slot_count, x, common);
  for (uint64_t r = 0; r < n_regions; ++r) {
    child_box(box, n, &s, r, cb);
    feasible[r] = (uint8_t)inc_child(p, box, cb, common, var_ids, slot_count, x, xs, &obj_lb[r], &obj_ub[r]);
  }
  free(xs);
  free(x);
  free(common);
  free(cb);
  return 0;
}

/* ======================================================================
 * batched algorithm, restated step for step from the device solver
 * ==================================================================== */
/* Total order on lower bounds used by parent selection and eviction: the
 * IEEE bit pattern mapped to an unsigned key (NaN sorts after +inf). */
static inline uint64_t lb_key(double x)
{
  uint64_t u = dbits(x);
  if (x != x) return UINT64_MAX;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}

typedef struct {
  uint64_t key;
  uint64_t pos;
} keypos;

static int keypos_cmp(const void* a, const void* b)
{
  const keypos* x = (const keypos*)a;
  const keypos* y = (const keypos*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->pos < y->pos ? -1 : (x->pos > y->pos ? 1 : 0);
}

typedef struct {
  double* box; /* cap x 2n */
  double* lb;
  uint32_t* depth;
  uint64_t n, cap;
} pool_t;

static void pool_reserve(pool_t* P, uint64_t cap, int64_t nv)
{
  if (cap <= P->cap) return;
  P->box = (double*)realloc(P->box, sizeof(double) * 2 * (size_t)nv * cap);
  P->lb = (double*)realloc(P->lb, sizeof(double) * cap);
  P->depth = (uint32_t*)realloc(P->depth, sizeof(uint32_t) * cap);
  P->cap = cap;
}

typedef struct {
  uint8_t kinds[64];
  uint64_t vids[64], widths[64], dom[64];
  int64_t count;
  uint64_t nreg;
  int fathom;
  slots_t s;
} parent_plan;

typedef struct {
  const orc_problem* p;
  const cmn_solve_options* o;
  const double* pbox; /* E x 2n */
  const parent_plan* plan;
  uint64_t C; /* child slots per parent */
  uint64_t E;
  double gub_old;
  uint64_t salt0;
  int use_screen; /* FP32 screen switched on for this iteration */
  const double* plb; /* lazy form: the parents' FP64 lower bounds */
  const float* common; /* lazy form, incremental: [parent][segment] (lo, hi) */
  /* outputs per child slot (E*C) */
  double* lb;
  uint8_t* state; /* 0 invalid, 1 dup, 2 infeasible, 3 dominated(old), 4 eligible */
  uint8_t* screened; /* FP32 screen excluded it */
  double* cand_val;  /* per child slot: best candidate value (inf none) */
  int64_t* cand_idx; /* element index within parent */
  float* b32v;       /* lazy form: per child slot, smallest FP32 point value */
  uint32_t* b32i;    /* and its sample index */
  int failed;
} batch_ctx;

/* Lazy form: survivors whose FP32 bound lies within LAZY_BAND *
 * max(1, |GUB|) below the incumbent are certified in FP64 when bounded
 * (kCertifyBand in csrc/kernels.cuh). */
#define LAZY_BAND (1.0 / 1024.0)

/* Lazy form, incremental children: each parent's common chain sums. */
typedef struct {
  const orc_problem* p;
  const double* pbox;
  const parent_plan* plan;
  float* common;
} common_ctx;

static void common_range(void* vc, int64_t k0, int64_t k1, int tid)
{
  (void)tid;
  common_ctx* c = (common_ctx*)vc;
  const orc_problem* p = c->p;
  iv32* x = (iv32*)malloc(sizeof(iv32) * (size_t)(p->n_vars ? p->n_vars : 1));
  for (int64_t k = k0; k < k1; ++k) {
    if (c->plan[k].nreg == 0) continue;
    inc_common_one(p, c->pbox + 2 * (size_t)p->n_vars * (size_t)k, c->plan[k].vids, c->plan[k].count, x,
                   c->common + 2 * (size_t)p->inc_segments * (size_t)k);
  }
  free(x);
}

/* Lazy form: the FP64 verdict of each selected parent box. */
typedef struct {
  const orc_problem* p;
  const double* pbox;
  double* lb;
  int* feas;
  int failed;
} certify_ctx;

static void certify_range(void* vc, int64_t k0, int64_t k1, int tid)
{
  (void)tid;
  certify_ctx* c = (certify_ctx*)vc;
  const int64_t n = c->p->n_vars;
  iv64* slots = (iv64*)malloc(sizeof(iv64) * (size_t)(c->p->n_prog_slots > 0 ? c->p->n_prog_slots : 1));
  for (int64_t k = k0; k < k1; ++k) {
    double ub;
    const int f = program_run64(c->p, c->pbox + 2 * (size_t)n * (size_t)k, slots, &c->lb[k], &ub, 1);
    if (f < 0) c->failed = 1;
    c->feas[k] = f > 0;
  }
  free(slots);
}

/* One child slot: interval bound (FP64, or FP32 screen + FP64 certify, or
 * FP32 alone in the lazy form) and then its samples (or its exact point
 * for a fathomed parent). */
static void batch_range(void* vc, int64_t g0, int64_t g1, int tid)
{
  (void)tid;
  batch_ctx* c = (batch_ctx*)vc;
  const orc_problem* p = c->p;
  const int64_t n = p->n_vars;
  double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* x = (double*)malloc(sizeof(double) * (size_t)n);
  iv64* v64 = (iv64*)malloc(sizeof(iv64) * (size_t)p->n_nodes);
  iv32* v32 = (iv32*)malloc(sizeof(iv32) * (size_t)p->n_nodes);
  iv32* xs = (iv32*)malloc(sizeof(iv32) * (size_t)(n ? n : 1));
  double* pv = (double*)malloc(sizeof(double) * (size_t)p->n_nodes);
  float* pf = (float*)malloc(sizeof(float) * (size_t)p->n_nodes);
  const int lazy = c->o->precision == CMN_PRECISION_FP32_LAZY;
  for (int64_t g = g0; g < g1; ++g) {
    uint64_t k = (uint64_t)g / c->C, r = (uint64_t)g % c->C;
    const parent_plan* pl = &c->plan[k];
    c->cand_val[g] = INFINITY;
    c->cand_idx[g] = -1;
    c->screened[g] = 0;
    if (lazy) {
      c->b32v[g] = INFINITY;
      c->b32i[g] = 0;
    }
    if (r >= pl->nreg) {
      c->state[g] = 0;
      c->lb[g] = NAN;
      continue;
    }
    const double* parent = c->pbox + 2 * (size_t)n * k;
    child_box(parent, n, &pl->s, r, cb);
    if (pl->fathom) {
      /* exact enumeration point (graph/kernels.cuh:131-172) */
      for (int64_t v = 0; v < n; ++v) x[v] = cb[2 * v];
      c->state[g] = 0;
      c->lb[g] = NAN;
      if (lazy) { /* screened in FP32 like a sample; verified per chunk */
        float o32;
        int f32 = eval_point_f(p, x, pf, &o32);
        float v32 = (f32 && o32 == o32) ? o32 : INFINITY;
        if (v32 < c->b32v[g]) c->b32v[g] = v32;
        continue;
      }
      double obj;
      int f = eval_point_impl(p, x, pv, &obj);
      if (f && witness_is_admissible(p, x)) {
        c->cand_val[g] = obj;
        c->cand_idx[g] = (int64_t)r;
      } else if (f && obj < c->gub_old) {
        c->cand_idx[g] = -2; /* feasible but inadmissible witness */
        c->cand_val[g] = obj;
      }
      continue;
    }
    if (is_dup(r, &pl->s, pl->dom)) {
      c->state[g] = 1;
      c->lb[g] = NAN;
    } else {
      double lb, ub;
      int f, screened_out = 0;
      if (c->o->precision == CMN_PRECISION_FP32_LAZY) {
        /* FP32; the parent's certified FP64 bound holds for the child; a
         * survivor within the band below the incumbent is certified in
         * FP64 at once (csrc/kernels.cuh certify_floor) */
        if (c->common) {
          f = inc_child(p, parent, cb, c->common + 2 * (size_t)p->inc_segments * k, pl->vids, pl->count,
                        (iv32*)v32, xs, &lb, &ub);
        } else {
          if (eval_all_f(p, cb, v32)) c->failed = 1;
          f = verdict_f(p, v32, &lb, &ub);
        }
        double plb = c->plb[k];
        lb = plb > lb ? plb : lb;
        if (!f) {
          c->state[g] = 2;
        } else if (lb > c->gub_old) {
          c->state[g] = 3;
        } else if (lb >= c->gub_old - LAZY_BAND * fmax(1.0, fabs(c->gub_old))) {
          if (eval_all_d(p, cb, v64)) c->failed = 1;
          f = verdict_d(p, v64, &lb, &ub);
          lb = plb > lb ? plb : lb;
          c->state[g] = !f ? 2 : (lb > c->gub_old ? 3 : 4);
          c->screened[g] = 2; /* certified */
        } else {
          c->state[g] = 4;
        }
        screened_out = 1; /* no further FP64 pass */
      } else if (c->o->precision == CMN_PRECISION_FP32_SCREEN && c->use_screen) {
        if (eval_all_f(p, cb, v32)) c->failed = 1;
        f = verdict_f(p, v32, &lb, &ub);
        if (!f) {
          screened_out = 1;
          c->state[g] = 2;
        } else if (lb > c->gub_old) {
          screened_out = 1;
          c->state[g] = 3;
        }
        c->screened[g] = (uint8_t)screened_out;
      }
      if (!screened_out) {
        if (eval_all_d(p, cb, v64)) c->failed = 1;
        f = verdict_d(p, v64, &lb, &ub);
        c->state[g] = !f ? 2 : (lb > c->gub_old ? 3 : 4);
      }
      c->lb[g] = lb;
    }
    int do_sample = c->o->sample_all ? 1 : (c->state[g] == 4);
    if (do_sample && lazy) {
      uint64_t salt = c->salt0 + k + 1;
      for (uint64_t i = 0; i < c->o->sample_points; ++i) {
        sample_point(p, cb, r, i, salt, x);
        float o32;
        int f32 = eval_point_f(p, x, pf, &o32);
        float v32 = (f32 && o32 == o32) ? o32 : INFINITY;
        if (v32 < c->b32v[g]) {
          c->b32v[g] = v32;
          c->b32i[g] = (uint32_t)i;
        }
      }
    } else if (do_sample) {
      uint64_t salt = c->salt0 + k + 1;
      for (uint64_t i = 0; i < c->o->sample_points; ++i) {
        sample_point(p, cb, r, i, salt, x);
        double obj;
        int f = eval_point_impl(p, x, pv, &obj);
        double masked = f ? obj : INFINITY;
        int64_t idx = (int64_t)(r * c->o->sample_points + i);
        if (masked < c->cand_val[g]) {
          c->cand_val[g] = masked;
          c->cand_idx[g] = idx;
        }
      }
    }
  }
  free(cb);
  free(x);
  free(v64);
  free(v32);
  free(xs);
  free(pv);
  free(pf);
}

typedef struct {
  pool_t P;
  double GUB, GLB;
  int have_best;
  drop_acc dropped;
  uint64_t expansions, iterations;
  int converged, stopped_early, stop;
  int use_screen; /* FP32 screen on for the next iteration */
} bstate;

/* Runs the batched search for at most `max_iter` iterations (0 = no cap
 * beyond the options).  Returns -1 on evaluation failure. */
static int batched_run(const orc_problem* p, const cmn_solve_options* o,
                       uint64_t max_iter, bstate* st, cmn_counters* ct,
                       double* best_point, int threads)
{
  const int64_t n = p->n_vars;
  const uint64_t C = (uint64_t)1 << o->bisection_budget;
  const uint64_t S = o->sample_points;
  uint64_t cap = o->frontier_cap ? o->frontier_cap : (1ull << 20);
  if (o->precision == CMN_PRECISION_FP32_LAZY && !p->prog64) {
    set_err("the lazy form's verdict needs the FP64 program (orc_set_program64)");
    return -1;
  }
  double* x = (double*)malloc(sizeof(double) * (size_t)n);
  int rc = 0;
  uint64_t run_iters = 0;

  for (;;) {
    pool_t* P = &st->P;
    if (P->n == 0) break;
    double m = INFINITY;
    uint64_t mkey = UINT64_MAX;
    for (uint64_t i = 0; i < P->n; ++i) {
      uint64_t k = lb_key(P->lb[i]);
      if (k < mkey) {
        mkey = k;
        m = P->lb[i];
      }
    }
    if (gap_closed(st->GUB, m, o->tolerance)) {
      st->converged = 1;
      st->stop = CMN_STOP_CONVERGED;
      st->stopped_early = 1;
      break;
    }
    st->GLB = m;
    if (st->expansions >= o->iter_limit) break;
    if (o->batch_iter_limit && st->iterations >= o->batch_iter_limit) break;
    if (max_iter && run_iters >= max_iter) break;
    ++run_iters;
    ++st->iterations;

    uint64_t E = P->n;
    if (E > o->batch_parents) E = o->batch_parents;
    if (E > o->iter_limit - st->expansions) E = o->iter_limit - st->expansions;

    /* select the E best (key, position); parents keep pool order */
    keypos* kp = (keypos*)malloc(sizeof(keypos) * P->n);
    for (uint64_t i = 0; i < P->n; ++i) {
      kp[i].key = lb_key(P->lb[i]);
      kp[i].pos = i;
    }
    qsort(kp, P->n, sizeof(keypos), keypos_cmp);
    uint8_t* sel = (uint8_t*)calloc(P->n, 1);
    for (uint64_t i = 0; i < E; ++i) sel[kp[i].pos] = 1;
    free(kp);
    double* pbox = (double*)malloc(sizeof(double) * 2 * (size_t)n * E);
    uint32_t* pdepth = (uint32_t*)malloc(sizeof(uint32_t) * E);
    parent_plan* plan = (parent_plan*)malloc(sizeof(parent_plan) * E);
    uint64_t k = 0;
    for (uint64_t i = 0; i < P->n; ++i) {
      if (!sel[i]) continue;
      memcpy(pbox + 2 * (size_t)n * k, P->box + 2 * (size_t)n * i, sizeof(double) * 2 * (size_t)n);
      pdepth[k] = P->depth[i];
      ++k;
    }
    for (k = 0; k < E; ++k) {
      parent_plan* pl = &plan[k];
      const double* b = pbox + 2 * (size_t)n * k;
      pl->count = orc_bisection_choose(b, p->kinds, n, o->bisection_budget,
                                       (int64_t)o->max_cycle_size, (int64_t)o->enumerate_cap,
                                       o->relative_width, pl->kinds, pl->vids, pl->widths,
                                       pl->dom);
      int64_t live = 0;
      for (int64_t v = 0; v < n; ++v)
        if (b[2 * v + 1] > b[2 * v]) ++live;
      pl->nreg = pl->count == 0 ? 1 : slot_product(pl->widths, pl->count);
      pl->fathom = live <= pl->count && fully_enumerable(pl->kinds, pl->count);
      slots_init(&pl->s, pl->kinds, pl->vids, pl->widths, pl->count);
    }
    /* lazy form: a selected box is expanded only if its FP64 verdict
     * keeps it (the reference predicate, and its bound at most GUB) */
    double* plb = NULL;
    if (o->precision == CMN_PRECISION_FP32_LAZY) {
      plb = (double*)malloc(sizeof(double) * (E ? E : 1));
      int* pfeas = (int*)malloc(sizeof(int) * (E ? E : 1));
      certify_ctx cc = {p, pbox, plb, pfeas, 0};
      parallel_for((int64_t)E, threads, certify_range, &cc);
      if (cc.failed) {
        set_err("op without an interval implementation");
        rc = -1;
      }
      for (k = 0; k < E; ++k) {
        ++ct->certified_fp64;
        if (!pfeas[k] || plb[k] > st->GUB) {
          plan[k].nreg = 0;
          plan[k].fathom = 0;
          plan[k].count = 0;
          ++ct->certify_pruned;
        }
      }
      free(pfeas);
    }
    uint64_t salt0 = st->expansions;
    st->expansions += E;

    uint64_t G = E * C;
    batch_ctx c;
    memset(&c, 0, sizeof c);
    c.p = p;
    c.o = o;
    c.pbox = pbox;
    c.plan = plan;
    c.C = C;
    c.E = E;
    c.gub_old = st->GUB;
    c.salt0 = salt0;
    c.use_screen = st->use_screen;
    c.plb = plb;
    float* common = NULL;
    if (o->precision == CMN_PRECISION_FP32_LAZY && p->inc_ok) {
      common = (float*)malloc(sizeof(float) * 2 * (size_t)(p->inc_segments ? p->inc_segments : 1) * (E ? E : 1));
      common_ctx cc = {p, pbox, plan, common};
      parallel_for((int64_t)E, threads, common_range, &cc);
      c.common = common;
    }
    c.lb = (double*)malloc(sizeof(double) * G);
    c.state = (uint8_t*)malloc(G);
    c.screened = (uint8_t*)malloc(G);
    c.cand_val = (double*)malloc(sizeof(double) * G);
    c.cand_idx = (int64_t*)malloc(sizeof(int64_t) * G);
    const int lazy = o->precision == CMN_PRECISION_FP32_LAZY;
    c.b32v = lazy ? (float*)malloc(sizeof(float) * G) : NULL;
    c.b32i = lazy ? (uint32_t*)malloc(sizeof(uint32_t) * G) : NULL;
    parallel_for((int64_t)G, threads, batch_range, &c);
    if (c.failed) {
      set_err("op without an interval implementation");
      rc = -1;
    }
    if (lazy) {
      /* each chunk of 32 child slots: its FP32-best point (first child,
       * then first sample, on ties) evaluated again in FP64 */
      double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)n);
      double* val = (double*)malloc(sizeof(double) * (size_t)p->n_nodes);
      for (uint64_t c0 = 0; c0 < G; c0 += 32) {
        float bv = INFINITY;
        uint64_t bg = 0;
        for (uint64_t g = c0; g < c0 + 32 && g < G; ++g)
          if (c.b32v[g] < bv) {
            bv = c.b32v[g];
            bg = g;
          }
        if (!(bv < INFINITY)) continue;
        uint64_t kk = bg / C, r = bg % C, i = c.b32i[bg];
        const parent_plan* pl = &plan[kk];
        child_box(pbox + 2 * (size_t)n * kk, n, &pl->s, r, cb);
        if (pl->fathom) {
          for (int64_t v = 0; v < n; ++v) x[v] = cb[2 * v];
        } else {
          sample_point(p, cb, r, i, salt0 + kk + 1, x);
        }
        double obj;
        int f = eval_point_impl(p, x, val, &obj);
        if (!f || obj != obj) continue;
        if (pl->fathom && !witness_is_admissible(p, x)) {
          if (obj < st->GUB) {
            c.cand_idx[bg] = -2;
            c.cand_val[bg] = obj;
          }
          continue;
        }
        c.cand_val[bg] = obj;
        c.cand_idx[bg] = (int64_t)(pl->fathom ? r : r * S + i);
      }
      free(cb);
      free(val);
    }

    /* incumbent: argmin over (value, parent, element) of admissible
     * feasible candidates */
    uint64_t iter_valid = 0, iter_excluded = 0, iter_certified = 0;
    double best = INFINITY;
    uint64_t best_k = 0;
    int64_t best_e = -1;
    for (k = 0; k < E; ++k) {
      const parent_plan* pl = &plan[k];
      if (pl->fathom) {
        ++ct->fathomed;
        ct->fathomed_points += pl->nreg;
      } else {
        ct->bounded += pl->nreg;
      }
      for (uint64_t r = 0; r < C; ++r) {
        uint64_t g = k * C + r;
        if (r >= pl->nreg) continue;
        if (!pl->fathom) {
          if (c.state[g] != 1) { /* duplicates are never evaluated */
            ++iter_valid;
            if (c.state[g] == 2 || c.state[g] == 3) ++iter_excluded;
            if (o->precision == CMN_PRECISION_FP32_LAZY) {
              ++ct->screened_fp32;
              if (c.screened[g] == 2) ++ct->certified_fp64;
            } else if (o->precision == CMN_PRECISION_FP32_SCREEN && st->use_screen) {
              ++ct->screened_fp32;
              if (!c.screened[g]) {
                ++ct->certified_fp64;
                ++iter_certified;
              }
            } else {
              ++ct->certified_fp64;
              ++iter_certified;
            }
          }
          if (o->sample_all || c.state[g] == 4) ct->sampled += S;
        }
        if (c.cand_idx[g] == -2) {
          ++ct->witness_rejected;
          continue;
        }
        if (c.cand_idx[g] < 0) continue;
        double v = c.cand_val[g];
        if (v < best) {
          best = v;
          best_k = k;
          best_e = c.cand_idx[g];
        }
      }
    }
    if (best_e >= 0 && best < st->GUB) {
      const parent_plan* pl = &plan[best_k];
      const double* parent = pbox + 2 * (size_t)n * best_k;
      double* cb = (double*)malloc(sizeof(double) * 2 * (size_t)n);
      if (pl->fathom) {
        child_box(parent, n, &pl->s, (uint64_t)best_e, cb);
        for (int64_t v = 0; v < n; ++v) x[v] = cb[2 * v];
      } else {
        uint64_t r = (uint64_t)best_e / S, i = (uint64_t)best_e % S;
        child_box(parent, n, &pl->s, r, cb);
        sample_point(p, cb, r, i, salt0 + best_k + 1, x);
      }
      free(cb);
      st->GUB = best;
      memcpy(best_point, x, sizeof(double) * (size_t)n);
      st->have_best = 1;
    }
    /* the screen stays on while it excludes >= 1/4 of the children it sees
     * and comes back once the FP64 verdicts would have excluded 1/4 */
    if (o->precision == CMN_PRECISION_FP32_SCREEN && iter_valid > 0) {
      uint64_t x = st->use_screen ? iter_valid - iter_certified : iter_excluded;
      st->use_screen = x * 4 >= iter_valid;
    }
    double gub = st->GUB;

    /* prune with the new incumbent and rebuild the pool: unselected
     * entries in pool order, then kept children in (parent, region) order */
    uint64_t kept = 0;
    for (uint64_t g = 0; g < G; ++g) {
      uint8_t s = c.state[g];
      if (s == 0) continue;
      if (s == 1) ++ct->pruned_duplicate;
      else if (s == 2) ++ct->pruned_infeasible;
      else if (s == 3 || c.lb[g] > gub) ++ct->pruned_dominated;
      else ++kept;
    }
    uint64_t remaining = P->n - E;
    pool_t NP;
    memset(&NP, 0, sizeof NP);
    pool_reserve(&NP, remaining + kept + 1, n);
    for (uint64_t i = 0; i < P->n; ++i) {
      if (sel[i]) continue;
      memcpy(NP.box + 2 * (size_t)n * NP.n, P->box + 2 * (size_t)n * i, sizeof(double) * 2 * (size_t)n);
      NP.lb[NP.n] = P->lb[i];
      NP.depth[NP.n] = P->depth[i];
      ++NP.n;
    }
    for (uint64_t g = 0; g < G; ++g) {
      if (c.state[g] != 4 || c.lb[g] > gub) continue;
      uint64_t kk = g / C, r = g % C;
      child_box(pbox + 2 * (size_t)n * kk, n, &plan[kk].s, r, NP.box + 2 * (size_t)n * NP.n);
      NP.lb[NP.n] = c.lb[g];
      NP.depth[NP.n] = pdepth[kk] + 1;
      ++NP.n;
    }
    ct->enqueued += kept;
    /* eviction above the cap: keep the `cap` best (key, position) */
    if (NP.n > cap) {
      keypos* kq = (keypos*)malloc(sizeof(keypos) * NP.n);
      for (uint64_t i = 0; i < NP.n; ++i) {
        kq[i].key = lb_key(NP.lb[i]);
        kq[i].pos = i;
      }
      qsort(kq, NP.n, sizeof(keypos), keypos_cmp);
      uint8_t* keep = (uint8_t*)calloc(NP.n, 1);
      for (uint64_t i = 0; i < cap; ++i) keep[kq[i].pos] = 1;
      free(kq);
      uint64_t w = 0;
      for (uint64_t i = 0; i < NP.n; ++i) {
        if (!keep[i]) {
          drop_fold(&st->dropped, NP.lb[i], gub);
          continue;
        }
        if (w != i) {
          memcpy(NP.box + 2 * (size_t)n * w, NP.box + 2 * (size_t)n * i, sizeof(double) * 2 * (size_t)n);
          NP.lb[w] = NP.lb[i];
          NP.depth[w] = NP.depth[i];
        }
        ++w;
      }
      NP.n = w;
      free(keep);
    }
    ct->dropped_viable = st->dropped.viable;
    ct->dropped_dominated = st->dropped.dominated;
    free(P->box);
    free(P->lb);
    free(P->depth);
    *P = NP;
    if (P->n > ct->peak_frontier) ct->peak_frontier = P->n;
    free(sel);
    free(pbox);
    free(pdepth);
    free(plan);
    free(plb);
    free(c.lb);
    free(c.state);
    free(c.screened);
    free(c.cand_val);
    free(c.cand_idx);
    free(c.b32v);
    free(c.b32i);
    free(common);
    if (rc) break;
  }
  free(x);
  return rc;
}

static void batched_init(const orc_problem* p, const cmn_solve_options* o,
                         bstate* st)
{
  memset(st, 0, sizeof *st);
  const int64_t n = p->n_vars;
  pool_reserve(&st->P, 1, n);
  for (int64_t v = 0; v < n; ++v) {
    st->P.box[2 * v] = p->var_lb[v];
    st->P.box[2 * v + 1] = p->var_ub[v];
  }
  st->P.lb[0] = -DBL_MAX;
  st->P.depth[0] = 0;
  st->P.n = 1;
  st->GUB = o->has_known_primal ? o->known_primal_bound : DBL_MAX;
  st->GLB = -DBL_MAX;
  st->dropped.lb_min = INFINITY;
  st->stop = CMN_STOP_ITERATION_LIMIT;
  st->use_screen = 1;
}

static void batched_finish(const orc_problem* p, const cmn_solve_options* o,
                           bstate* st, cmn_outcome* out, double* best_point)
{
  cmn_counters ct = out->counters;
  if (!st->stopped_early)
    st->stop = st->P.n == 0 ? CMN_STOP_EXHAUSTED
               : gap_closed(st->GUB, st->GLB, o->tolerance) ? CMN_STOP_CONVERGED
                                                            : CMN_STOP_ITERATION_LIMIT;
  int found = st->GUB < DBL_MAX;
  uint64_t viable = 0;
  double fmin_lb = DBL_MAX;
  uint64_t mkey = UINT64_MAX;
  for (uint64_t i = 0; i < st->P.n; ++i) {
    if (st->P.lb[i] <= st->GUB) ++viable;
    uint64_t k = lb_key(st->P.lb[i]);
    if (k < mkey) {
      mkey = k;
      fmin_lb = st->P.lb[i];
    }
  }
  finalise(st->GLB, st->GUB, o->tolerance, found, st->converged, st->P.n == 0, fmin_lb,
           viable, &st->dropped, out);
  out->upper_bound = st->GUB;
  out->stop_reason = st->stop;
  out->found_incumbent = found;
  out->frontier_size = st->P.n;
  out->viable = viable;
  out->dropped_lb_min = st->dropped.lb_min;
  ct.iterations = st->iterations;
  ct.expansions = st->expansions;
  out->counters = ct;
  if (!st->have_best)
    for (int64_t v = 0; v < p->n_vars; ++v) best_point[v] = NAN;
}

int orc_solve_batched(const orc_problem* p, const cmn_solve_options* opts,
                      cmn_outcome* out, double* best_point, int threads)
{
  cmn_solve_options o;
  opts_norm(opts, &o);
  memset(out, 0, sizeof *out);
  out->counters.peak_frontier = 1; /* the root box */
  bstate st;
  batched_init(p, &o, &st);
  int rc = batched_run(p, &o, 0, &st, &out->counters, best_point, threads);
  batched_finish(p, &o, &st, out, best_point);
  free(st.P.box);
  free(st.P.lb);
  free(st.P.depth);
  return rc;
}

int64_t orc_batched_frontier(const orc_problem* p,
                             const cmn_solve_options* opts,
                             uint64_t iterations, double* pool_box,
                             double* pool_lb, uint32_t* pool_depth,
                             int64_t pool_room, cmn_outcome* out,
                             double* best_point, int threads)
{
  cmn_solve_options o;
  opts_norm(opts, &o);
  memset(out, 0, sizeof *out);
  out->counters.peak_frontier = 1; /* the root box */
  bstate st;
  batched_init(p, &o, &st);
  int rc = batched_run(p, &o, iterations, &st, &out->counters, best_point, threads);
  batched_finish(p, &o, &st, out, best_point);
  int64_t count = (int64_t)st.P.n;
  int64_t m = count < pool_room ? count : pool_room;
  const int64_t n = p->n_vars;
  if (pool_box) memcpy(pool_box, st.P.box, sizeof(double) * 2 * (size_t)n * (size_t)m);
  if (pool_lb) memcpy(pool_lb, st.P.lb, sizeof(double) * (size_t)m);
  if (pool_depth) memcpy(pool_depth, st.P.depth, sizeof(uint32_t) * (size_t)m);
  free(st.P.box);
  free(st.P.lb);
  free(st.P.depth);
  return rc ? -1 : count;
}
