/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the SQUANDER (rakytap/sequential-quantum-gate-decomposer)
 * decomposition hot path: parametric-circuit application to a 2^n x cols complex128
 * matrix, the FROBENIUS_NORM / HILBERT_SCHMIDT_TEST / INFIDELITY cost functions and
 * their gradients, the batched cost, and the BFGS (Powell-Z) and ADAM decomposition drivers.
 *
 * It is the checker for the CUDA engine (tests, smoke(), the CPU-baseline leg of
 * bench.py).  Nothing in the engine links or calls it.  Every routine follows the
 * reference algorithm step by step, including its summation order and its
 * "(1 - tr/N) - 1" gradient formula, so that parity can be checked against the
 * reference's own arithmetic.  Reference citations are paths inside the
 * SQUANDER tree (src-cpp = squander/src-cpp).
 *
 * Memory layout (as the reference Matrix, src-cpp/common/include/QGDTypes.h:33-38 and
 * matrix_base.hpp:38-59): row-major interleaved complex128 {re, im} with a row stride
 * counted in complex elements.  Qubit q is bit q of the row index (LSB = qubit 0),
 * src-cpp/gates/kernels/apply_kernel_to_input.cpp:52-67.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Gate type ids as in src-cpp/gates/include/Gate.h:37-50. */
enum { T_CZ = 4, T_CNOT = 5, T_U3 = 7, T_RY = 8, T_RX = 9, T_RZ = 10, T_CRY = 14 };

typedef struct {
  int type, target, control, param_start;
} sqgo_gate;

/* Number of free parameters per gate: U3 = 3 (U3.cpp:31), RX/RY/RZ/CRY = 1
 * (RY.cpp:8, CRY inherits RY), CNOT/CZ = 0. */
static int param_num(int type) {
  switch (type) {
    case T_U3: return 3;
    case T_RX: case T_RY: case T_RZ: case T_CRY: return 1;
    default: return 0;
  }
}

int sqgo_gate_param_num(int type) { return param_num(type); }

/* 2x2 gate kernel k[0..7] = {u00, u01, u10, u11} as (re, im) from the per-parameter
 * (sin, cos) of the STORED parameter value (Gates_block.cpp:269-279 precomputes
 * sin/cos of the stored value; U3 stores theta/2, U3.cpp:49-51).  deriv_param >= 0
 * selects the derivative kernel with respect to that parameter.
 *   U3: gate_kernel_templates.h:509-521 (forward), :555-603 (d/dtheta, d/dphi, d/dlambda)
 *   RX: :193-199 / :226-232;  RY: :237-243 / :265-271;  RZ: :281-287 / :309-315.
 * Returns 0 for an invalid request. */
static int gate_kernel(int type, const double* sc, int deriv_param, double k[8]) {
  memset(k, 0, 8 * sizeof(double));
  if (type == T_U3) {
    double st = sc[0], ct = sc[1], sp = sc[2], cp = sc[3], sl = sc[4], cl = sc[5];
    double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
    if (deriv_param < 0) {
      k[0] = ct;        k[1] = 0;
      k[2] = -st * cl;  k[3] = -st * sl;
      k[4] = st * cp;   k[5] = st * sp;
      k[6] = ct * cpl;  k[7] = ct * spl;
    } else if (deriv_param == 0) {
      k[0] = -st;       k[1] = 0;
      k[2] = -ct * cl;  k[3] = -ct * sl;
      k[4] = ct * cp;   k[5] = ct * sp;
      k[6] = -st * cpl; k[7] = -st * spl;
    } else if (deriv_param == 1) {
      k[4] = -st * sp;  k[5] = st * cp;
      k[6] = -ct * spl; k[7] = ct * cpl;
    } else if (deriv_param == 2) {
      k[2] = st * sl;   k[3] = -st * cl;
      k[6] = -ct * spl; k[7] = ct * cpl;
    } else {
      return 0;
    }
    return 1;
  }
  double s = sc[0], c = sc[1];
  if (deriv_param > 0) return 0;
  if (deriv_param == 0) {
    /* The one-parameter derivative kernels (gate_kernel_templates.h:226-232, 265-271,
     * 309-315) are the forward forms with s -> cos and c -> -sin. */
    double t = s; s = c; c = -t;
  }
  switch (type) {
    case T_RX:
      k[0] = c; k[3] = -s; k[5] = -s; k[6] = c; return 1;
    case T_RY: case T_CRY:
      k[0] = c; k[2] = -s; k[4] = s; k[6] = c; return 1;
    case T_RZ:
      k[0] = c; k[1] = -s; k[6] = c; k[7] = s; return 1;
    default: return 0;
  }
}

/* Left-apply of a (controlled) 2x2 kernel, apply_kernel_to_input.cpp:34-115:
 * rows (i, i + 2^t) with bit t of i clear; when a control is given only rows whose
 * control bit is set are transformed; with deriv != 0 the untransformed row pairs
 * are zeroed (the derivative of the identity block). */
static void apply_kernel(double* m, int rows, int cols, int stride, const double* k, int target, int control,
                         int deriv) {
  const int step = 1 << target;
  for (int base = 0; base + step < rows; base += step << 1) {
    for (int idx = 0; idx < step; idx++) {
      int i = base + idx, j = i + step;
      double* x = m + 2L * i * stride;
      double* y = m + 2L * j * stride;
      if (control < 0 || ((i >> control) & 1)) {
        for (int col = 0; col < cols; col++) {
          double xr = x[2 * col], xi = x[2 * col + 1], yr = y[2 * col], yi = y[2 * col + 1];
          double t1r = k[0] * xr - k[1] * xi, t1i = k[0] * xi + k[1] * xr;
          double t2r = k[2] * yr - k[3] * yi, t2i = k[2] * yi + k[3] * yr;
          x[2 * col] = t1r + t2r;
          x[2 * col + 1] = t1i + t2i;
          t1r = k[4] * xr - k[5] * xi; t1i = k[4] * xi + k[5] * xr;
          t2r = k[6] * yr - k[7] * yi; t2i = k[6] * yi + k[7] * yr;
          y[2 * col] = t1r + t2r;
          y[2 * col + 1] = t1i + t2i;
        }
      } else if (deriv) {
        memset(x, 0, 16L * cols);
        memset(y, 0, 16L * cols);
      }
    }
  }
}

/* Right-apply M <- M * G, apply_kernel_to_input.cpp:131-178 (column pairs). */
static void apply_kernel_right(double* m, int rows, int cols, int stride, const double* k, int target, int control) {
  const int step = 1 << target;
  for (int r = 0; r < rows; r++) {
    double* row = m + 2L * r * stride;
    for (int base = 0; base + step < cols; base += step << 1) {
      for (int idx = 0; idx < step; idx++) {
        int i = base + idx, j = i + step;
        if (control >= 0 && !((i >> control) & 1)) continue;
        double xr = row[2 * i], xi = row[2 * i + 1], yr = row[2 * j], yi = row[2 * j + 1];
        double t1r = k[0] * xr - k[1] * xi, t1i = k[0] * xi + k[1] * xr;
        double t2r = k[4] * yr - k[5] * yi, t2i = k[4] * yi + k[5] * yr;
        row[2 * i] = t1r + t2r;
        row[2 * i + 1] = t1i + t2i;
        t1r = k[2] * xr - k[3] * xi; t1i = k[2] * xi + k[3] * xr;
        t2r = k[6] * yr - k[7] * yi; t2i = k[6] * yi + k[7] * yr;
        row[2 * j] = t1r + t2r;
        row[2 * j + 1] = t1i + t2i;
      }
    }
  }
}

/* CNOT: swap row pairs whose control bit is set,
 * apply_dedicated_gate_kernel_to_input.cpp:46-93.  CZ: negate the target=1 row of
 * pairs whose control bit is set, :221-254. */
static void apply_x(double* m, int rows, int cols, int stride, int target, int control) {
  const int step = 1 << target;
  for (int base = 0; base + step < rows; base += step << 1)
    for (int idx = 0; idx < step; idx++) {
      int i = base + idx, j = i + step;
      if (control >= 0 && !((i >> control) & 1)) continue;
      double* x = m + 2L * i * stride;
      double* y = m + 2L * j * stride;
      for (int c = 0; c < 2 * cols; c++) { double t = x[c]; x[c] = y[c]; y[c] = t; }
    }
}
static void apply_z(double* m, int rows, int cols, int stride, int target, int control) {
  const int step = 1 << target;
  for (int base = 0; base + step < rows; base += step << 1)
    for (int idx = 0; idx < step; idx++) {
      int i = base + idx, j = i + step;
      if (control >= 0 && !((i >> control) & 1)) continue;
      double* y = m + 2L * j * stride;
      for (int c = 0; c < 2 * cols; c++) y[c] = -y[c];
    }
}
/* Right-apply of CNOT swaps column pairs, of CZ negates columns. */
static void apply_x_right(double* m, int rows, int cols, int stride, int target, int control) {
  const int step = 1 << target;
  for (int r = 0; r < rows; r++) {
    double* row = m + 2L * r * stride;
    for (int base = 0; base + step < cols; base += step << 1)
      for (int idx = 0; idx < step; idx++) {
        int i = base + idx, j = i + step;
        if (control >= 0 && !((i >> control) & 1)) continue;
        double t0 = row[2 * i], t1 = row[2 * i + 1];
        row[2 * i] = row[2 * j]; row[2 * i + 1] = row[2 * j + 1];
        row[2 * j] = t0; row[2 * j + 1] = t1;
      }
  }
}
static void apply_z_right(double* m, int rows, int cols, int stride, int target, int control) {
  const int step = 1 << target;
  for (int r = 0; r < rows; r++) {
    double* row = m + 2L * r * stride;
    for (int base = 0; base + step < cols; base += step << 1)
      for (int idx = 0; idx < step; idx++) {
        int i = base + idx, j = i + step;
        if (control >= 0 && !((i >> control) & 1)) continue;
        row[2 * j] = -row[2 * j]; row[2 * j + 1] = -row[2 * j + 1];
      }
  }
}

/* sin/cos of every stored parameter, Gates_block.cpp:269-279 (std::sin, std::cos). */
static double* precompute_sincos(const double* params, int P) {
  double* sc = (double*)malloc(sizeof(double) * 2 * (P > 0 ? P : 1));
  for (int p = 0; p < P; p++) { sc[2 * p] = sin(params[p]); sc[2 * p + 1] = cos(params[p]); }
  return sc;
}

/* Gate::apply_to_inner (Gate.cpp:549-570) / Gate::apply_kernel_to (Gate.cpp:1478-1768)
 * dispatch for one gate, forward (deriv_param < 0) or derivative kernel. */
static void apply_gate(const sqgo_gate* g, const double* sc, double* m, int rows, int cols, int stride, int deriv_param) {
  double k[8];
  switch (g->type) {
    case T_CNOT: apply_x(m, rows, cols, stride, g->target, g->control); return;
    case T_CZ: apply_z(m, rows, cols, stride, g->target, g->control); return;
    case T_U3: case T_RX: case T_RY: case T_RZ:
      gate_kernel(g->type, sc + 2 * g->param_start, deriv_param, k);
      apply_kernel(m, rows, cols, stride, k, g->target, -1, deriv_param >= 0);
      return;
    case T_CRY:
      gate_kernel(g->type, sc + 2 * g->param_start, deriv_param, k);
      apply_kernel(m, rows, cols, stride, k, g->target, g->control, deriv_param >= 0);
      return;
  }
}

static int check_gates(int qbit_num, const sqgo_gate* g, int L, int P) {
  int p = 0;
  for (int i = 0; i < L; i++) {
    int t = g[i].type;
    if (t != T_CZ && t != T_CNOT && t != T_U3 && t != T_RY && t != T_RX && t != T_RZ && t != T_CRY) return -1;
    if (g[i].target < 0 || g[i].target >= qbit_num) return -2;
    if ((t == T_CZ || t == T_CNOT || t == T_CRY) && (g[i].control < 0 || g[i].control >= qbit_num || g[i].control == g[i].target))
      return -3;
    if (g[i].param_start != p) return -4;
    p += param_num(t);
  }
  return p == P ? 0 : -5;
}

/* Gates_block::apply_to / apply_to_inner, Gates_block.cpp:606-710 (unfused branch):
 * gates[0] is applied first. */
int sqgo_apply_to(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, double* m, int rows, int cols,
                  int stride) {
  if (rows != (1 << qbit_num)) return -10;
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  double* sc = precompute_sincos(params, P);
  for (int i = 0; i < L; i++) apply_gate(&g[i], sc, m, rows, cols, stride, -1);
  free(sc);
  return 0;
}

/* Gates_block::apply_from_right, Gates_block.cpp:885-935: M <- M * C where
 * C = G_{L-1} ... G_0, i.e. gates are right-applied from the last one back. */
int sqgo_apply_from_right(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, double* m, int rows,
                          int cols, int stride) {
  if (cols != (1 << qbit_num)) return -10;
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  double* sc = precompute_sincos(params, P);
  for (int i = L - 1; i >= 0; i--) {
    double k[8];
    switch (g[i].type) {
      case T_CNOT: apply_x_right(m, rows, cols, stride, g[i].target, g[i].control); break;
      case T_CZ: apply_z_right(m, rows, cols, stride, g[i].target, g[i].control); break;
      default:
        gate_kernel(g[i].type, sc + 2 * g[i].param_start, -1, k);
        apply_kernel_right(m, rows, cols, stride, k, g[i].target, g[i].type == T_CRY ? g[i].control : -1);
    }
  }
  free(sc);
  return 0;
}

/* Gates_block::apply_derivate_to, prefix branch (Gates_block.cpp:1012-1150 with
 * build_forward_inputs :430-470 and Gate::apply_derivative_to_precomputed
 * Gate.cpp:645-706): for every parameter of gate k, copy the forward input of gate
 * k, apply the derivative kernel (zeroing uncontrolled rows), then apply gates
 * k+1..L-1.  out holds P matrices rows x cols (stride cols). */
int sqgo_apply_derivate_to(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, const double* in,
                           int rows, int cols, int stride, double* out) {
  if (rows != (1 << qbit_num)) return -10;
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  double* sc = precompute_sincos(params, P);
  size_t msz = (size_t)rows * cols * 2;
  double* fwd = (double*)malloc(sizeof(double) * msz);
  for (int r = 0; r < rows; r++) memcpy(fwd + 2L * r * cols, in + 2L * r * stride, 16L * cols);
  for (int i = 0; i < L; i++) {
    int pn = param_num(g[i].type);
    for (int p = 0; p < pn; p++) {
      double* d = out + msz * (g[i].param_start + p);
      memcpy(d, fwd, sizeof(double) * msz);
      apply_gate(&g[i], sc, d, rows, cols, cols, p);
      for (int j = i + 1; j < L; j++) apply_gate(&g[j], sc, d, rows, cols, cols, -1);
    }
    apply_gate(&g[i], sc, fwd, rows, cols, cols, -1);
  }
  free(fwd);
  free(sc);
  return 0;
}

/* Cost variants (Optimization_Interface.h:43-45). */
enum { FROBENIUS_NORM = 0, HILBERT_SCHMIDT_TEST = 3, INFIDELITY = 9 };

/* get_cost_function, N_Qubit_Decomposition_Cost_Function.cpp:73-162: sequential sum of
 * Re M[idx + offset, idx] over idx < cols. */
static double real_trace(const double* m, int cols, int stride, int off) {
  double t = 0.0;
  for (int idx = 0; idx < cols; idx++) t += m[2L * ((long)(idx + off) * stride + idx)];
  return t;
}
/* get_trace, N_Qubit_Decomposition_Cost_Function.cpp:482-499 (no trace offset). */
static void complex_trace(const double* m, int cols, int stride, double* tr, double* ti) {
  double a = 0.0, b = 0.0;
  for (int idx = 0; idx < cols; idx++) {
    a += m[2L * ((long)idx * stride + idx)];
    b += m[2L * ((long)idx * stride + idx) + 1];
  }
  *tr = a; *ti = b;
}

/* Optimization_Interface::calculate_cost_function, Optimization_Interface.cpp:677-735. */
double sqgo_cost_of_matrix(const double* m, int cols, int stride, int trace_offset, int variant) {
  if (variant == FROBENIUS_NORM) return 1.0 - real_trace(m, cols, stride, trace_offset) / cols;
  double tr, ti;
  complex_trace(m, cols, stride, &tr, &ti);
  if (variant == HILBERT_SCHMIDT_TEST) {
    double d = 1.0 / cols;
    return 1.0 - d * d * (tr * tr + ti * ti);
  }
  if (variant == INFIDELITY) {
    double d = cols;
    return 1.0 - ((tr * tr + ti * ti) / d + 1) / (d + 1);
  }
  return NAN;
}

/* Optimization_Interface::optimization_problem, Optimization_Interface.cpp:634-668. */
int sqgo_cost(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, const double* target, int cols,
              int trace_offset, int variant, double* cost) {
  int rows = 1 << qbit_num;
  double* m = (double*)malloc(16L * rows * cols);
  memcpy(m, target, 16L * rows * cols);
  int rc = sqgo_apply_to(qbit_num, g, L, params, P, m, rows, cols, cols);
  if (!rc) *cost = sqgo_cost_of_matrix(m, cols, cols, trace_offset, variant);
  free(m);
  return rc;
}

/* Optimization_Interface::optimization_problem_combined_non_static, CPU branch
 * Optimization_Interface.cpp:1379-1472: apply_to_combined then, per parameter,
 * FROBENIUS: get_cost_function(dM) - 1;  HS: -2 d^2 (Re t Re dt + Im t Im dt);
 * INFIDELITY: -2/d/(d+1) (Re t Re dt + Im t Im dt). */
int sqgo_cost_grad(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, const double* target,
                   int cols, int trace_offset, int variant, double* cost, double* grad) {
  int rows = 1 << qbit_num;
  size_t msz = (size_t)rows * cols * 2;
  double* m = (double*)malloc(sizeof(double) * msz);
  double* d = (double*)malloc(sizeof(double) * msz * (P > 0 ? P : 1));
  memcpy(m, target, sizeof(double) * msz);
  int rc = sqgo_apply_derivate_to(qbit_num, g, L, params, P, target, rows, cols, cols, d);
  if (!rc) rc = sqgo_apply_to(qbit_num, g, L, params, P, m, rows, cols, cols);
  if (!rc) {
    *cost = sqgo_cost_of_matrix(m, cols, cols, trace_offset, variant);
    double tr = 0, ti = 0;
    if (variant != FROBENIUS_NORM) complex_trace(m, cols, cols, &tr, &ti);
    for (int p = 0; p < P; p++) {
      const double* dm = d + msz * p;
      if (variant == FROBENIUS_NORM) {
        grad[p] = sqgo_cost_of_matrix(dm, cols, cols, trace_offset, FROBENIUS_NORM) - 1.0;
      } else {
        double dr, di;
        complex_trace(dm, cols, cols, &dr, &di);
        if (variant == HILBERT_SCHMIDT_TEST) {
          double dd = 1.0 / cols;
          grad[p] = -2.0 * dd * dd * tr * dr - 2.0 * dd * dd * ti * di;
        } else {
          double dd = cols;
          grad[p] = -2.0 / dd / (dd + 1) * tr * dr - 2.0 / dd / (dd + 1) * ti * di;
        }
      }
    }
  }
  free(m);
  free(d);
  return rc;
}

/* ---------------- gradient by a reverse sweep (sizes the prefix form cannot hold) -----
 * The reference materialises all P derivative matrices (Gates_block.cpp:1012-1150),
 * which needs P * 16 * rows * cols bytes: 30 GB at 10 qubits with 1830 parameters.  This
 * is the same gradient, organised so that it needs three matrices:
 *   t_p = sum_{i<cols} (S_j dG_j P_j)[i + off, i] = sum_{i, a, b} R_j[i, a] dG_j[a, b] P_j[b, i]
 * with P_j = G_{j-1}..G_0 T (rows x cols, the input of gate j) and R_j = E G_{L-1}..G_{j+1}
 * (cols x rows, E selecting rows off..off+cols-1).  The sweep starts from W = C T and
 * R = E and walks the gates backwards: P_j = G_j^dagger P_{j+1} (uncomputation, exact up
 * to rounding because the gates are unitary), R_{j-1} = R_j G_j.  dG_j is the derivative
 * kernel with the reference's zeroing of uncontrolled row pairs (apply_kernel_to_input.cpp:93-97).
 * The gradient formulas are those of sqgo_cost_grad.  It agrees with the prefix form to
 * rounding; the tests check both against the reference where both fit in memory. */
static void kernel_dagger(const double* k, double* kd) {
  kd[0] = k[0]; kd[1] = -k[1]; kd[2] = k[4]; kd[3] = -k[5];
  kd[4] = k[2]; kd[5] = -k[3]; kd[6] = k[6]; kd[7] = -k[7];
}

/* sum_i sum_{a,b} R[i,a] D[a,b] P[b,i] for the embedded derivative kernel D of one gate */
static void deriv_contract(const double* R, const double* Pm, int rows, int cols, const double* k, int target,
                           int control, double* out_r, double* out_i) {
  const int step = 1 << target;
  double sr = 0.0, si = 0.0;
  for (int base = 0; base + step < rows; base += step << 1) {
    for (int idx = 0; idx < step; idx++) {
      int r0 = base + idx, r1 = r0 + step;
      if (control >= 0 && !((r0 >> control) & 1)) continue;
      const double* p0 = Pm + 2L * r0 * cols;
      const double* p1 = Pm + 2L * r1 * cols;
      for (int i = 0; i < cols; i++) {
        double ar = p0[2 * i], ai = p0[2 * i + 1], br = p1[2 * i], bi = p1[2 * i + 1];
        /* (D P)[r0, i] and (D P)[r1, i] */
        double xr = k[0] * ar - k[1] * ai + k[2] * br - k[3] * bi;
        double xi = k[0] * ai + k[1] * ar + k[2] * bi + k[3] * br;
        double yr = k[4] * ar - k[5] * ai + k[6] * br - k[7] * bi;
        double yi = k[4] * ai + k[5] * ar + k[6] * bi + k[7] * br;
        const double* q = R + 2L * i * rows;
        double u0r = q[2 * r0], u0i = q[2 * r0 + 1], u1r = q[2 * r1], u1i = q[2 * r1 + 1];
        sr += u0r * xr - u0i * xi + u1r * yr - u1i * yi;
        si += u0r * xi + u0i * xr + u1r * yi + u1i * yr;
      }
    }
  }
  *out_r = sr;
  *out_i = si;
}

int sqgo_cost_grad_sweep(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, const double* target,
                         int cols, int trace_offset, int variant, double* cost, double* grad) {
  int rows = 1 << qbit_num;
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  size_t msz = (size_t)rows * cols * 2;
  double* Pm = (double*)malloc(sizeof(double) * msz);
  double* R = (double*)calloc(msz, sizeof(double));
  memcpy(Pm, target, sizeof(double) * msz);
  rc = sqgo_apply_to(qbit_num, g, L, params, P, Pm, rows, cols, cols);
  if (rc) { free(Pm); free(R); return rc; }
  *cost = sqgo_cost_of_matrix(Pm, cols, cols, trace_offset, variant);
  double tr = 0, ti = 0;
  if (variant != FROBENIUS_NORM) complex_trace(Pm, cols, cols, &tr, &ti);
  const int off = variant == FROBENIUS_NORM ? trace_offset : 0;
  for (int i = 0; i < cols; i++) R[2L * ((size_t)i * rows + i + off)] = 1.0;
  double* sc = precompute_sincos(params, P);
  for (int j = L - 1; j >= 0; j--) {
    const sqgo_gate* gj = &g[j];
    double k[8], kd[8];
    /* P <- G_j^dagger P */
    switch (gj->type) {
      case T_CNOT: apply_x(Pm, rows, cols, cols, gj->target, gj->control); break;
      case T_CZ: apply_z(Pm, rows, cols, cols, gj->target, gj->control); break;
      default:
        gate_kernel(gj->type, sc + 2 * gj->param_start, -1, k);
        kernel_dagger(k, kd);
        apply_kernel(Pm, rows, cols, cols, kd, gj->target, gj->type == T_CRY ? gj->control : -1, 0);
    }
    int pn = param_num(gj->type);
    for (int p = 0; p < pn; p++) {
      double dk[8], dr, di;
      gate_kernel(gj->type, sc + 2 * gj->param_start, p, dk);
      deriv_contract(R, Pm, rows, cols, dk, gj->target, gj->type == T_CRY ? gj->control : -1, &dr, &di);
      double* gp = &grad[gj->param_start + p];
      if (variant == FROBENIUS_NORM) {
        *gp = (1.0 - dr / cols) - 1.0;
      } else if (variant == HILBERT_SCHMIDT_TEST) {
        double dd = 1.0 / cols;
        *gp = -2.0 * dd * dd * tr * dr - 2.0 * dd * dd * ti * di;
      } else {
        double dd = cols;
        *gp = -2.0 / dd / (dd + 1) * tr * dr - 2.0 / dd / (dd + 1) * ti * di;
      }
    }
    /* R <- R G_j */
    switch (gj->type) {
      case T_CNOT: apply_x_right(R, cols, rows, rows, gj->target, gj->control); break;
      case T_CZ: apply_z_right(R, cols, rows, rows, gj->target, gj->control); break;
      default:
        apply_kernel_right(R, cols, rows, rows, k, gj->target, gj->type == T_CRY ? gj->control : -1);
    }
  }
  free(sc);
  free(Pm);
  free(R);
  return 0;
}

/* ---------------- thread-parallel batch (Optimization_Interface.cpp:940-1033) ------- */
typedef struct {
  int qbit_num, L, P, cols, trace_offset, variant, with_grad, B, tstride, sweep;
  const sqgo_gate* g;
  const double* params;
  const double* target;
  double* cost;
  double* grad;
  int next;
  pthread_mutex_t mu;
  int rc;
} batch_job;

static void* batch_worker(void* arg) {
  batch_job* j = (batch_job*)arg;
  size_t tsz = (size_t)2 * (1 << j->qbit_num) * j->cols;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    int b = j->next++;
    pthread_mutex_unlock(&j->mu);
    if (b >= j->B) break;
    const double* tgt = j->target + (j->tstride ? tsz * b : 0);
    int rc;
    if (j->with_grad && j->sweep)
      rc = sqgo_cost_grad_sweep(j->qbit_num, j->g, j->L, j->params + (size_t)b * j->P, j->P, tgt, j->cols,
                                j->trace_offset, j->variant, &j->cost[b], j->grad + (size_t)b * j->P);
    else if (j->with_grad)
      rc = sqgo_cost_grad(j->qbit_num, j->g, j->L, j->params + (size_t)b * j->P, j->P, tgt, j->cols, j->trace_offset,
                          j->variant, &j->cost[b], j->grad + (size_t)b * j->P);
    else
      rc = sqgo_cost(j->qbit_num, j->g, j->L, j->params + (size_t)b * j->P, j->P, tgt, j->cols, j->trace_offset,
                     j->variant, &j->cost[b]);
    if (rc) j->rc = rc;
  }
  return NULL;
}

/* Batched cost (and optional gradient) of B parameter vectors.  target_per_instance
 * selects one target per instance (B x rows x cols) instead of one shared target; sweep
 * selects the reverse-sweep gradient (sqgo_cost_grad_sweep) instead of the prefix form. */
int sqgo_batch2(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, int B, const double* target,
                int cols, int target_per_instance, int trace_offset, int variant, double* cost, double* grad,
                int nthreads, int sweep) {
  batch_job j;
  memset(&j, 0, sizeof(j));
  j.qbit_num = qbit_num; j.L = L; j.P = P; j.cols = cols; j.trace_offset = trace_offset; j.variant = variant;
  j.with_grad = grad != NULL; j.B = B; j.tstride = target_per_instance; j.g = g; j.params = params; j.target = target;
  j.cost = cost; j.grad = grad; j.sweep = sweep;
  pthread_mutex_init(&j.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  pthread_t th[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &j);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&j.mu);
  return j.rc;
}

int sqgo_batch(int qbit_num, const sqgo_gate* g, int L, const double* params, int P, int B, const double* target,
               int cols, int target_per_instance, int trace_offset, int variant, double* cost, double* grad,
               int nthreads) {
  return sqgo_batch2(qbit_num, g, L, params, P, B, target, cols, target_per_instance, trace_offset, variant, cost,
                     grad, nthreads, 0);
}

/* ---------------- BFGS (Powell Z-matrix) decomposition driver ----------------------
 * src-cpp/common/BFGS_Powell.cpp:70-192 (Optimize), :202-396 (BFGS_iteration),
 * :407-446 (get_search_direction); src-cpp/common/grad_descend.cpp:127-273
 * (line_search), :399-425 (get_Maximal_Line_Search_Step); restarts and outer loop
 * from optimization_engines/BFGS.cpp:42-152 and Decomposition_Base.cpp:375-700. */
typedef struct {
  int qbit_num, L, P, cols, trace_offset, variant;
  const sqgo_gate* g;
  const double* target;
  long calls;
} fg_ctx;

static void fg_eval(fg_ctx* c, const double* x, double* f, double* grad) {
  c->calls++;
  sqgo_cost_grad(c->qbit_num, c->g, c->L, x, c->P, c->target, c->cols, c->trace_offset, c->variant, f, grad);
}

static const double NUM_PRECISION = 1.42e-14; /* grad_descend.cpp:37 */

static void search_direction(int n, const double* Z, const double* g, double* ztg, double* d, double* overlap) {
  for (int c = 0; c < n; c++) ztg[c] = 0.0;
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++) ztg[c] += Z[(long)r * n + c] * g[r];
  for (int r = 0; r < n; r++) {
    d[r] = 0.0;
    for (int c = 0; c < n; c++) d[r] = d[r] - Z[(long)r * n + c] * ztg[c];
  }
  double o = 0.0;
  for (int i = 0; i < n; i++) o += d[i] * g[i];
  *overlap = o;
}

static void bfgs_update(int n, double* Z, double* ztg, const double* x, const double* g, const double* x0,
                        const double* g0, double* norm_Z, double* work) {
  double* delta = work;
  double* gamma = work + n;
  double* gTz = work + 2 * n;
  double* nz = work + 3 * n;
  double norm_delta = 0.0, dtg = 0.0, tmp = 0.0;
  for (int i = 0; i < n; i++) {
    delta[i] = x[i] - x0[i];
    norm_delta += delta[i] * delta[i];
    tmp += g0[i] * delta[i];
    gamma[i] = g[i] - g0[i];
    dtg += gamma[i] * delta[i];
  }
  if (dtg < fabs(tmp) * 0.1) return;
  dtg = fmax(NUM_PRECISION, dtg);
  for (int col = n - 1; col > 0; col--) {
    if (ztg[col] == 0.0) continue;
    int cm = col - 1;
    double a = sqrt(ztg[cm] * ztg[cm] + ztg[col] * ztg[col]);
    double cv = ztg[cm] / a, sv = ztg[col] / a;
    ztg[cm] = a;
    long off = cm;
    for (int r = 0; r < n; r++) {
      double t = cv * Z[off + 1] - sv * Z[off];
      Z[off] = cv * Z[off] + sv * Z[off + 1];
      Z[off + 1] = t;
      off += n;
    }
  }
  if (*norm_Z < 0.0) {
    *norm_Z = norm_delta / dtg;
  } else {
    tmp = sqrt(*norm_Z * norm_delta / dtg);
    *norm_Z = fmin(*norm_Z, tmp);
    *norm_Z = fmax(*norm_Z, tmp * 0.1);
  }
  tmp = sqrt(dtg);
  for (int i = 0; i < n; i++) Z[(long)i * n] = fabs(delta[i]) > NUM_PRECISION ? delta[i] / tmp : 0.0;
  for (int c = 0; c < n; c++) gTz[c] = 0.0;
  for (int r = 0; r < n; r++)
    for (int c = 1; c < n; c++) gTz[c] += gamma[r] * Z[(long)r * n + c];
  for (int c = 1; c < n; c++) gTz[c] = gTz[c] / dtg;
  for (int c = 0; c < n; c++) nz[c] = 0.0;
  for (int r = 0; r < n; r++)
    for (int c = 1; c < n; c++) {
      double* z = &Z[(long)r * n + c];
      *z = *z - gTz[c] * delta[r];
      nz[c] += *z * *z;
    }
  for (int c = 1; c < n; c++) {
    if (nz[c] < *norm_Z && nz[c] > NUM_PRECISION) {
      tmp = sqrt(*norm_Z / nz[c]);
      for (int r = 0; r < n; r++) Z[(long)r * n + c] *= tmp;
    }
  }
}

/* Returns the final cost; x is updated in place.  max_calls bounds cost+gradient
 * evaluations (maximal_iterations of the reference). */
static double bfgs_powell(fg_ctx* c, double* x, long max_calls) {
  int n = c->P;
  double* Z = (double*)calloc((size_t)n * n, sizeof(double));
  double* buf = (double*)malloc(sizeof(double) * 12 * n);
  double *g = buf, *d = buf + n, *x0 = buf + 2 * n, *g0 = buf + 3 * n, *ztg = buf + 4 * n, *gbest = buf + 5 * n,
         *work = buf + 6 * n;
  for (int i = 0; i < n; i++) Z[(long)i * n + i] = 1.0;
  double norm_Z = -1.0, f;
  c->calls = 0;
  fg_eval(c, x, &f, g);
  double fprev = fabs(f + f + 1.0);
  for (;;) {
    double max_step = 0.0, dg = 0.0;
    search_direction(n, Z, g, ztg, d, &dg);
    if (dg < 0.0) {
      for (int k = 0; k < n; k++) {
        if (fabs(d[k]) < 1e-5) continue;
        double b = fabs(2 * M_PI / d[k]);
        if (max_step == 0.0 || b < max_step) max_step = b;
      }
    }
    double gn = 0.0;
    for (int i = 0; i < n; i++) gn += g[i] * g[i];
    if (gn <= 1e-19 * 1e-19) break;
    if (dg >= 0.0) break;
    if (f >= fprev) break;
    fprev = f;
    if (c->calls >= max_calls) break;
    /* line search, grad_descend.cpp:127-273 */
    memcpy(x0, x, sizeof(double) * n);
    memcpy(g0, g, sizeof(double) * n);
    memcpy(gbest, g, sizeof(double) * n);
    double step = fmin(1.0, max_step);
    double f_low = f, f_high = f, s_high = max_step, s_low = 0.0, s_best = 0.0, f_best = f, dg_best = fabs(dg);
    double dg_high = 0.0;
    for (int it = 0; it < 50; it++) {
      for (int i = 0; i < n; i++) x[i] = x0[i] + step * d[i];
      fg_eval(c, x, &f, g);
      double dgc = 0.0;
      for (int i = 0; i < n; i++) dgc += d[i] * g[i];
      if (f < f_best || fabs(dgc) < dg_best) {
        s_best = step; f_best = f; dg_best = fabs(dgc);
        memcpy(gbest, g, sizeof(double) * n);
      }
      if (c->calls == max_calls) break;
      if (f < f_low + step * 0.1 * dg) {
        if (dgc >= dg * 0.7) break;
        s_low = step; f_low = f;
      } else {
        s_high = step; f_high = f; dg_high = dgc;
      }
      if (it == 0 || s_low > 0.0) {
        double dlf = (f_high - f_low) / (s_high - s_low) * 2.0 - dg_high;
        double scale = -dlf * 0.5 / (dg_high - dlf);
        scale = fmax(0.1, scale);
        step = s_low + scale * (s_high - s_low);
      } else {
        step = step * 0.1;
        if (step < NUM_PRECISION) break;
      }
    }
    if (step != s_best) {
      step = s_best; f = f_best;
      memcpy(g, gbest, sizeof(double) * n);
      for (int i = 0; i < n; i++) x[i] = x0[i] + step * d[i];
    }
    if (step == 0.0) break;
    bfgs_update(n, Z, ztg, x, g, x0, g0, &norm_Z, work);
  }
  free(Z);
  free(buf);
  return f;
}

static uint64_t splitmix(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* Counter-based uniform draw in [0, 1): the splitmix64 finaliser of k (53 random bits).
 * The engine draws its restart perturbations the same way, so that decompositions with
 * restarts can be compared draw for draw. */
static double counter_u01(uint64_t k) {
  uint64_t z = k + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* N_Qubit_Decomposition_custom::start_decomposition (N_Qubit_Decomposition_custom.cpp:116-190)
 * with BFGS (chosen for qbit_num <= 5, :59-76): up to max_outer outer iterations, each
 * running iteration_loops BFGS_Powell restarts (BFGS.cpp:121-150); after an improved
 * minimum the guess is perturbed by U[0, 2 pi)/100; the loop stops once the minimum is
 * below the tolerance (Decomposition_Base.cpp:742-752).  The reference draws the
 * perturbation from std::mt19937; here draw i of a perturbation is counter_u01(ctr + i),
 * with ctr starting at `counter` and advancing by (P + 1) * (2^32 + 1) per perturbation. */
int sqgo_decompose(int qbit_num, const sqgo_gate* g, int L, int P, const double* target, int cols, int trace_offset,
                   int variant, double* x, double tolerance, long max_inner, int max_outer, int iteration_loops,
                   uint64_t counter, double* final_cost, long* total_calls) {
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  fg_ctx c = {qbit_num, L, P, cols, trace_offset, variant, g, target, 0};
  double* guess = (double*)malloc(sizeof(double) * P);
  memcpy(guess, x, sizeof(double) * P);
  double best = INFINITY;
  long calls = 0;
  uint64_t ctr = counter;
  for (int outer = 0; outer < max_outer; outer++) {
    for (int loop = 0; loop < iteration_loops; loop++) {
      double f = bfgs_powell(&c, guess, max_inner);
      calls += c.calls;
      if (best > f) {
        best = f;
        memcpy(x, guess, sizeof(double) * P);
        for (int i = 0; i < P; i++) guess[i] = x[i] + counter_u01(ctr + (uint64_t)i) * (2 * M_PI) / 100.0;
        ctr += 0x100000001ULL * (uint64_t)(P + 1);
      }
    }
    memcpy(guess, x, sizeof(double) * P);
    if (fabs(best) < tolerance) break;
  }
  free(guess);
  *final_cost = best;
  if (total_calls) *total_calls = calls;
  return 0;
}

typedef struct {
  int qbit_num, L, P, cols, trace_offset, variant, B, max_outer, iteration_loops;
  const sqgo_gate* g;
  const double* targets;
  double* x;
  double tolerance;
  long max_inner;
  uint64_t seed;
  double* cost;
  long* calls;
  int next;
  pthread_mutex_t mu;
} dec_job;

static void* dec_worker(void* arg) {
  dec_job* j = (dec_job*)arg;
  size_t tsz = (size_t)2 * (1 << j->qbit_num) * j->cols;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    int b = j->next++;
    pthread_mutex_unlock(&j->mu);
    if (b >= j->B) break;
    sqgo_decompose(j->qbit_num, j->g, j->L, j->P, j->targets + tsz * b, j->cols, j->trace_offset, j->variant,
                   j->x + (size_t)b * j->P, j->tolerance, j->max_inner, j->max_outer, j->iteration_loops,
                   j->seed * 0x2545F4914F6CDD1DULL + (uint64_t)b * 0x9E3779B97F4A7C15ULL, &j->cost[b],
                   &j->calls[b]);
  }
  return NULL;
}

/* B independent decompositions (one target each) spread over nthreads threads. */
int sqgo_decompose_batch(int qbit_num, const sqgo_gate* g, int L, int P, int B, const double* targets, int cols,
                         int trace_offset, int variant, double* x, double tolerance, long max_inner, int max_outer,
                         int iteration_loops, uint64_t seed, double* cost, long* calls, int nthreads) {
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  dec_job j;
  memset(&j, 0, sizeof(j));
  j.qbit_num = qbit_num; j.L = L; j.P = P; j.cols = cols; j.trace_offset = trace_offset; j.variant = variant;
  j.B = B; j.max_outer = max_outer; j.iteration_loops = iteration_loops; j.g = g; j.targets = targets; j.x = x;
  j.tolerance = tolerance; j.max_inner = max_inner; j.seed = seed; j.cost = cost; j.calls = calls;
  pthread_mutex_init(&j.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, dec_worker, &j);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&j.mu);
  return 0;
}

/* ---------------- ADAM decomposition driver ----------------------------------------
 * Optimization_Interface::solve_layer_optimization_problem_ADAM
 * (optimization_engines/ADAM.cpp:44-330) with Adam::update (common/Adam.cpp:138-270),
 * Adam::reset (:70-100), randomize_parameters (decomposition/Optimization_Interface.cpp:
 * 576-607), the settings of set_optimizer(ADAM) (:1625-1628: random_shift_count_max 100)
 * and the constructor defaults (adaptive_eta on, radius 1, randomization_rate 0.3, :56-64).
 * Adam's bias-correction powers advance once per parameter, in parameter order (the
 * reference advances them inside its parallel parameter loop).  Random numbers come from
 * the seeded splitmix64 stream of the BFGS driver (the reference uses std::mt19937). */
typedef struct {
  double beta1, beta2, eps, eta;
  double *mom, *var;
  double beta1_t, beta2_t;
  double f0_vec[100];
  double f0_mean;
  int f0_idx;
  int dec_vec[20];
  int dec_idx;
  double dec_test, f0_prev;
} adam_state;

static void adam_reset(adam_state* a, int P) {
  memset(a->mom, 0, sizeof(double) * P);
  memset(a->var, 0, sizeof(double) * P);
  a->beta1_t = 1.0;
  a->beta2_t = 1.0;
  memset(a->f0_vec, 0, sizeof(a->f0_vec));
  a->f0_mean = 0.0;
  a->f0_idx = 0;
  for (int i = 0; i < 20; i++) a->dec_vec[i] = -1;
  a->dec_idx = 0;
  a->dec_test = -1.0;
  a->f0_prev = DBL_MAX;
}

/* Returns 1 when the local-minimum test fires. */
static int adam_update(adam_state* a, double* x, const double* g, double f0, int P) {
  a->f0_mean = a->f0_mean + (f0 - a->f0_vec[a->f0_idx]) / 100;
  a->f0_vec[a->f0_idx] = f0;
  a->f0_idx = (a->f0_idx + 1) % 100;
  double var_f0 = 0.0;
  for (int i = 0; i < 100; i++) var_f0 = var_f0 + (a->f0_vec[i] - a->f0_mean) * (a->f0_vec[i] - a->f0_mean);
  var_f0 = sqrt(var_f0) / 100;
  if (f0 < a->f0_prev) {
    if (a->dec_vec[a->dec_idx] != 1) a->dec_test = a->dec_test + 2.0 / 20;
    a->dec_vec[a->dec_idx] = 1;
  } else {
    if (a->dec_vec[a->dec_idx] == 1) a->dec_test = a->dec_test - 2.0 / 20;
    a->dec_vec[a->dec_idx] = -1;
  }
  a->dec_idx = (a->dec_idx + 1) % 20;
  a->f0_prev = f0;
  double grad_var = 0.0;
  for (int i = 0; i < P; i++) grad_var += a->var[i];
  const int barren = grad_var < a->eps && a->dec_test > 0.7;
  const double eps = barren ? a->eps / 100 : a->eps;
  for (int i = 0; i < P; i++) {
    a->mom[i] = a->beta1 * a->mom[i] + (1 - a->beta1) * g[i];
    a->var[i] = a->beta2 * a->var[i] + (1 - a->beta2) * g[i] * g[i];
    a->beta1_t = a->beta1_t * a->beta1;
    const double mh = a->mom[i] / (1 - a->beta1_t);
    a->beta2_t = a->beta2_t * a->beta2;
    const double vh = a->var[i] / (1 - a->beta2_t);
    x[i] = x[i] - a->eta * mh / (sqrt(vh) + eps);
  }
  return (fabs(a->f0_mean - f0) < 1e-6 && a->dec_test <= 0.7 && var_f0 / a->f0_mean < 1e-6) ? 1 : 0;
}

int sqgo_adam_decompose(int qbit_num, const sqgo_gate* g, int L, int P, const double* target, int cols,
                        int trace_offset, int variant, double* x, double tolerance, long max_iters, double eta,
                        int adaptive_eta, int random_shift_count_max, long randomization_threshold, uint64_t seed,
                        double* final_cost, long* evals, long* nshifts) {
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  fg_ctx c = {qbit_num, L, P, cols, trace_offset, variant, g, target, 0};
  double* buf = (double*)malloc(sizeof(double) * 5 * (P > 0 ? P : 1));
  double *xt = buf, *best = buf + P, *grad = buf + 2 * P;
  adam_state a;
  a.beta1 = 0.68; a.beta2 = 0.8; a.eps = 1e-4; a.eta = eta;  /* Adam.cpp:31-40, ADAM.cpp eta default 1e-3 */
  a.mom = buf + 3 * P;
  a.var = buf + 4 * P;
  adam_reset(&a, P);
  memcpy(xt, x, sizeof(double) * P);
  memcpy(best, x, sizeof(double) * P);
  double current_minimum = DBL_MAX, hold = DBL_MAX, f0 = DBL_MAX;
  long sub_iter = 0, n = 0;
  int shifts = 0, status = 0;
  uint64_t s = seed;
  for (long it = 0; it < max_iters; it++) {
    fg_eval(&c, xt, &f0, grad);
    n++;
    if (sub_iter == 1) {
      hold = f0;
      if (adaptive_eta) a.eta = a.eta > 1e-3 ? a.eta : 1e-3;
    }
    if (hold * 0.95 > f0 || (hold * 0.97 > f0 && f0 < 1e-3) || (hold * 0.99 > f0 && f0 < 1e-4)) {
      sub_iter = 0;
      hold = f0;
    }
    if (current_minimum > f0) {
      current_minimum = f0;
      memcpy(best, xt, sizeof(double) * P);
      if (adaptive_eta) {  /* the second clamp overwrites the first, as in the reference */
        const double ne = 1e-3 * f0;
        a.eta = ne > 1e-6 ? ne : 1e-6;
        a.eta = ne < 1e-1 ? ne : 1e-1;
      }
    }
    if (f0 < tolerance || shifts > random_shift_count_max) break;
    if (sub_iter > randomization_threshold || status != 0) {
      sub_iter = 0;
      shifts++;
      hold = current_minimum;
      const double r = sqrt(f0);
      for (int j = 0; j < P; j++) {
        const double u = (double)(splitmix(&s) >> 11) * (1.0 / 9007199254740992.0);
        if (u <= 0.3) {
          const double w = (double)(splitmix(&s) >> 11) * (1.0 / 9007199254740992.0);
          xt[j] = best[j] + (-2 * M_PI + 4 * M_PI * w) * r * 1.0;
        } else {
          xt[j] = best[j];
        }
      }
      adam_reset(&a, P);
      status = 0;
    } else {
      status = adam_update(&a, xt, grad, f0, P);
    }
    sub_iter++;
  }
  memcpy(x, best, sizeof(double) * P);
  *final_cost = current_minimum;
  if (evals) *evals = n;
  if (nshifts) *nshifts = shifts;
  free(buf);
  return 0;
}

typedef struct {
  int qbit_num, L, P, cols, trace_offset, variant, B, adaptive_eta, random_shift_count_max;
  const sqgo_gate* g;
  const double* targets;
  double* x;
  double tolerance, eta;
  long max_iters, randomization_threshold;
  uint64_t seed;
  double* cost;
  long *evals, *shifts;
  int next;
  pthread_mutex_t mu;
} adam_job;

static void* adam_worker(void* arg) {
  adam_job* j = (adam_job*)arg;
  size_t tsz = (size_t)2 * (1 << j->qbit_num) * j->cols;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    int b = j->next++;
    pthread_mutex_unlock(&j->mu);
    if (b >= j->B) break;
    sqgo_adam_decompose(j->qbit_num, j->g, j->L, j->P, j->targets + tsz * b, j->cols, j->trace_offset, j->variant,
                        j->x + (size_t)b * j->P, j->tolerance, j->max_iters, j->eta, j->adaptive_eta,
                        j->random_shift_count_max, j->randomization_threshold, j->seed + (uint64_t)b * 7919u,
                        &j->cost[b], &j->evals[b], &j->shifts[b]);
  }
  return NULL;
}

/* B independent ADAM decompositions spread over nthreads threads (seed + 7919 b each). */
int sqgo_adam_batch(int qbit_num, const sqgo_gate* g, int L, int P, int B, const double* targets, int cols,
                    int trace_offset, int variant, double* x, double tolerance, long max_iters, double eta,
                    int adaptive_eta, int random_shift_count_max, long randomization_threshold, uint64_t seed,
                    double* cost, long* evals, long* shifts, int nthreads) {
  int rc = check_gates(qbit_num, g, L, P);
  if (rc) return rc;
  adam_job j;
  memset(&j, 0, sizeof(j));
  j.qbit_num = qbit_num; j.L = L; j.P = P; j.cols = cols; j.trace_offset = trace_offset; j.variant = variant;
  j.B = B; j.adaptive_eta = adaptive_eta; j.random_shift_count_max = random_shift_count_max; j.g = g;
  j.targets = targets; j.x = x; j.tolerance = tolerance; j.eta = eta; j.max_iters = max_iters;
  j.randomization_threshold = randomization_threshold; j.seed = seed; j.cost = cost; j.evals = evals;
  j.shifts = shifts;
  pthread_mutex_init(&j.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, adam_worker, &j);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&j.mu);
  return 0;
}
