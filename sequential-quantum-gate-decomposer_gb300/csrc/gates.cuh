// Device-side gate records, gate-matrix construction and the per-pair update rules
// shared by every kernel of the engine.
//
// FP64 is the scarce resource on GB300 (measured 1.2 TFLOP/s FMA, 1.05 TFLOP/s DMMA,
// against 6.7 TB/s HBM), so every rule here is written for the minimum number of FP64
// instructions: CNOT is a pure exchange, CZ a sign-bit flip done with integer logic,
// the one-parameter rotations use their real structure (8 FP64 ops per amplitude
// pair) and U3 uses its real (0,0) entry (14 ops per pair instead of 16).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sqg {

// Gate type ids of SQUANDER (src-cpp/gates/include/Gate.h:37-50).
enum : int { G_CZ = 4, G_CNOT = 5, G_U3 = 7, G_RY = 8, G_RX = 9, G_RZ = 10, G_CRY = 14 };
// Internal only (never in a caller's gate list): a general 2x2 unitary on one qubit, the product
// of a run of single-qubit gates in the merged forward plan (the id of SQUANDER's
// GENERAL_OPERATION).
enum : int { G_GEN = 1 };

struct Gate {
  int type, target, control, pstart;
};

__host__ __device__ inline int gate_param_num(int type) {
  return type == G_U3 ? 3 : (type == G_RX || type == G_RY || type == G_RZ || type == G_CRY) ? 1 : 0;
}
__host__ __device__ inline bool gate_controlled(int type) {
  return type == G_CNOT || type == G_CZ || type == G_CRY;
}

// Per-gate matrix record built once per parameter vector.  u[0..3] = u00, u01, u10,
// u11 of the 2x2 kernel (SQUANDER's gate_kernel_templates.h:193-287, 509-521); for the
// one-parameter rotations u[0] = (cos, sin) of the stored parameter and the structured
// rules below use only that.
struct GateMat {
  double2 u[4];
};

__device__ __forceinline__ double dneg(double v) {
  return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ULL);
}

// Row index of amplitude pair p for an uncontrolled gate on qubit t: p with a zero
// bit inserted at position t (the partner row is i | 2^t).
__device__ __forceinline__ int pair_index1(int p, int t) {
  return ((p >> t) << (t + 1)) | (p & ((1 << t) - 1));
}
// Row index of pair p for a gate on target t controlled by c: bit t = 0, bit c = 1.
__device__ __forceinline__ int pair_index2(int p, int t, int c) {
  int lo = t < c ? t : c, hi = t < c ? c : t;
  int i = ((p >> lo) << (lo + 1)) | (p & ((1 << lo) - 1));
  i = ((i >> hi) << (hi + 1)) | (i & ((1 << hi) - 1));
  return i | (1 << c);
}

// ---- per-pair update rules (x = row with target bit 0, y = partner row) ----------
// U3 with real u00: 14 FP64 instructions.
__device__ __forceinline__ void rule_u3(double2& x, double2& y, double u00, double2 u01, double2 u10, double2 u11) {
  double2 nx, ny;
  nx.x = fma(u00, x.x, fma(u01.x, y.x, -u01.y * y.y));
  nx.y = fma(u00, x.y, fma(u01.x, y.y, u01.y * y.x));
  ny.x = fma(u10.x, x.x, fma(-u10.y, x.y, fma(u11.x, y.x, -u11.y * y.y)));
  ny.y = fma(u10.x, x.y, fma(u10.y, x.x, fma(u11.x, y.y, u11.y * y.x)));
  x = nx;
  y = ny;
}
// General 2x2 [[u00, u01], [u10, u11]] with u00 = a + i s: 16 FP64 instructions.
__device__ __forceinline__ void rule_gen(double2& x, double2& y, double a, double s, double2 u01, double2 u10,
                                         double2 u11) {
  double2 nx, ny;
  nx.x = fma(a, x.x, fma(-s, x.y, fma(u01.x, y.x, -u01.y * y.y)));
  nx.y = fma(a, x.y, fma(s, x.x, fma(u01.x, y.y, u01.y * y.x)));
  ny.x = fma(u10.x, x.x, fma(-u10.y, x.y, fma(u11.x, y.x, -u11.y * y.y)));
  ny.y = fma(u10.x, x.y, fma(u10.y, x.x, fma(u11.x, y.y, u11.y * y.x)));
  x = nx;
  y = ny;
}
// RY / CRY [[c, -s], [s, c]]: 8 FP64 instructions.
__device__ __forceinline__ void rule_ry(double2& x, double2& y, double c, double s) {
  double2 nx, ny;
  nx.x = fma(c, x.x, -s * y.x);
  nx.y = fma(c, x.y, -s * y.y);
  ny.x = fma(s, x.x, c * y.x);
  ny.y = fma(s, x.y, c * y.y);
  x = nx;
  y = ny;
}
// RX [[c, -i s], [-i s, c]].
__device__ __forceinline__ void rule_rx(double2& x, double2& y, double c, double s) {
  double2 nx, ny;
  nx.x = fma(c, x.x, s * y.y);
  nx.y = fma(c, x.y, -s * y.x);
  ny.x = fma(c, y.x, s * x.y);
  ny.y = fma(c, y.y, -s * x.x);
  x = nx;
  y = ny;
}
// RZ diag(c - i s, c + i s).
__device__ __forceinline__ void rule_rz(double2& x, double2& y, double c, double s) {
  double2 nx, ny;
  nx.x = fma(c, x.x, s * x.y);
  nx.y = fma(c, x.y, -s * x.x);
  ny.x = fma(c, y.x, -s * y.y);
  ny.y = fma(c, y.y, s * y.x);
  x = nx;
  y = ny;
}

// Register copy of one gate's matrix, oriented for a forward (G), adjoint (G^dagger),
// transposed (G^T: right multiplication by G) or conjugated (conj G = (G^dagger)^T: right
// multiplication by G^dagger) update.
struct PairOp {
  int kind;  // G_U3, G_RY (also CRY), G_RX, G_RZ, G_CNOT, G_CZ, G_GEN
  double a;  // u00 (U3) or cos
  double s;  // sin (signed for adjoint)
  double2 b, c, d;  // u01, u10, u11 (U3)
};

enum Orientation { ORIENT_FWD = 0, ORIENT_ADJ = 1, ORIENT_TRANS = 2, ORIENT_CONJ = 3 };

// Sign flips go through dneg (an integer operation): a negated double that is stored,
// rather than folded into the consuming FMA, would cost an FP64 instruction per gate.
__device__ __forceinline__ PairOp make_op(int type, const GateMat& m, int orient) {
  PairOp op;
  op.kind = (type == G_CRY) ? G_RY : type;
  op.a = m.u[0].x;
  op.s = m.u[0].y;
  op.b = m.u[1];
  op.c = m.u[2];
  op.d = m.u[3];
  if (type == G_U3) {
    op.a = m.u[0].x;
    if (orient == ORIENT_ADJ) {  // [[u00, conj u10], [conj u01, conj u11]]
      op.b = make_double2(m.u[2].x, dneg(m.u[2].y));
      op.c = make_double2(m.u[1].x, dneg(m.u[1].y));
      op.d = make_double2(m.u[3].x, dneg(m.u[3].y));
    } else if (orient == ORIENT_TRANS) {  // [[u00, u10], [u01, u11]]
      op.b = m.u[2];
      op.c = m.u[1];
    } else if (orient == ORIENT_CONJ) {  // [[u00, conj u01], [conj u10, conj u11]]
      op.b = make_double2(m.u[1].x, dneg(m.u[1].y));
      op.c = make_double2(m.u[2].x, dneg(m.u[2].y));
      op.d = make_double2(m.u[3].x, dneg(m.u[3].y));
    }
  } else if (type == G_GEN) {
    // u00 = a + i s (op.a, op.s), u01 = b, u10 = c, u11 = d as stored
    if (orient == ORIENT_ADJ) {  // [[conj u00, conj u10], [conj u01, conj u11]]
      op.s = dneg(op.s);
      op.b = make_double2(m.u[2].x, dneg(m.u[2].y));
      op.c = make_double2(m.u[1].x, dneg(m.u[1].y));
      op.d = make_double2(m.u[3].x, dneg(m.u[3].y));
    } else if (orient == ORIENT_TRANS) {
      op.b = m.u[2];
      op.c = m.u[1];
    } else if (orient == ORIENT_CONJ) {
      op.s = dneg(op.s);
      op.b = make_double2(m.u[1].x, dneg(m.u[1].y));
      op.c = make_double2(m.u[2].x, dneg(m.u[2].y));
      op.d = make_double2(m.u[3].x, dneg(m.u[3].y));
    }
  } else if (type == G_RY || type == G_CRY) {
    // RY^dagger = RY^T = RY(-theta); RY is real, so conj RY = RY
    if (orient == ORIENT_ADJ || orient == ORIENT_TRANS) op.s = dneg(op.s);
  } else if (type == G_RX || type == G_RZ) {
    // RX, RZ are symmetric: RX^T = RX, RZ^T = RZ; adjoint and conjugate flip the sine.
    if (orient == ORIENT_ADJ || orient == ORIENT_CONJ) op.s = dneg(op.s);
  }
  return op;
}

__device__ __forceinline__ void apply_op(const PairOp& op, double2& x, double2& y) {
  switch (op.kind) {
    case G_U3: rule_u3(x, y, op.a, op.b, op.c, op.d); break;
    case G_GEN: rule_gen(x, y, op.a, op.s, op.b, op.c, op.d); break;
    case G_RY: rule_ry(x, y, op.a, op.s); break;
    case G_RX: rule_rx(x, y, op.a, op.s); break;
    case G_RZ: rule_rz(x, y, op.a, op.s); break;
    case G_CNOT: { double2 t = x; x = y; y = t; } break;
    case G_CZ: y.x = dneg(y.x); y.y = dneg(y.y); break;
  }
}

// Derivative kernel D of parameter k of a gate from the (sin, cos) of its stored
// parameters (SQUANDER gate_kernel_templates.h:226-232, 265-271, 309-315, 555-603).
__device__ __forceinline__ void deriv_kernel(int type, const double2* sc, int k, double2 D[4]) {
  if (type == G_U3) {
    double st = sc[0].x, ct = sc[0].y, sp = sc[1].x, cp = sc[1].y, sl = sc[2].x, cl = sc[2].y;
    double spl = sp * cl + cp * sl, cpl = cp * cl - sp * sl;
    if (k == 0) {
      D[0] = make_double2(-st, 0.0);
      D[1] = make_double2(-ct * cl, -ct * sl);
      D[2] = make_double2(ct * cp, ct * sp);
      D[3] = make_double2(-st * cpl, -st * spl);
    } else if (k == 1) {
      D[0] = make_double2(0.0, 0.0);
      D[1] = make_double2(0.0, 0.0);
      D[2] = make_double2(-st * sp, st * cp);
      D[3] = make_double2(-ct * spl, ct * cpl);
    } else {
      D[0] = make_double2(0.0, 0.0);
      D[1] = make_double2(st * sl, -st * cl);
      D[2] = make_double2(0.0, 0.0);
      D[3] = make_double2(-ct * spl, ct * cpl);
    }
    return;
  }
  double s0 = sc[0].x, c0 = sc[0].y;
  if (type == G_RX) {
    D[0] = make_double2(-s0, 0.0); D[1] = make_double2(0.0, -c0);
    D[2] = make_double2(0.0, -c0); D[3] = make_double2(-s0, 0.0);
  } else if (type == G_RZ) {
    D[0] = make_double2(-s0, -c0); D[1] = make_double2(0.0, 0.0);
    D[2] = make_double2(0.0, 0.0); D[3] = make_double2(-s0, c0);
  } else {  // RY, CRY
    D[0] = make_double2(-s0, 0.0); D[1] = make_double2(-c0, 0.0);
    D[2] = make_double2(c0, 0.0);  D[3] = make_double2(-s0, 0.0);
  }
}

}  // namespace sqg
