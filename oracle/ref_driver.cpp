/* ORACLE — test infrastructure only (never part of the engine).
 *
 * A C interface over SQUANDER's own C++ classes, compiled from the reference's sources
 * (oracle/build_ref.py) into oracle/_ref/libsqg_ref.so.  It lets the tests run the
 * reference itself on the same gate lists, parameters and targets that the oracle and the
 * CUDA engine see.  Each entry point states which reference call it makes:
 *
 *   sqgr_cost            N_Qubit_Decomposition_custom::optimization_problem
 *                        (squander/decomposition/qgd_N_Qubit_Decompositions_Wrapper.cpp:1396)
 *   sqgr_cost_grad       Optimization_Interface::optimization_problem_combined
 *                        (wrapper :1578, Optimization_Interface.cpp:1145-1485)
 *   sqgr_batch           Optimization_Interface::optimization_problem_batched
 *                        (wrapper :1650, Optimization_Interface.cpp:940-1033)
 *   sqgr_apply_to        Gates_block::apply_to (Gates_block.cpp:632-700)
 *   sqgr_apply_from_right Gates_block::apply_from_right (Gates_block.cpp:885-935)
 *   sqgr_apply_derivate_to Gates_block::apply_derivate_to (Gates_block.cpp:1012-1150)
 *   sqgr_combined_unitary Optimization_Interface::optimization_problem_combined_unitary
 *                        (wrapper :1446, Optimization_Interface.cpp:1525-1561)
 *   sqgr_tree_search     N_Qubit_Decomposition_Tree_Search::start_decomposition
 *                        (N_Qubit_Decomposition_Tree_Search.cpp, wrapper
 *                        qgd_N_Qubit_Decompositions_Wrapper.cpp:401-460): CNOT count and error found
 *   sqgr_bfgs_run        one BFGS_Powell::Start_Optimization run on
 *                        Optimization_Interface::optimization_problem_combined, as one
 *                        iteration of solve_layer_optimization_problem_BFGS makes it
 *                        (optimization_engines/BFGS.cpp:121-125, common/BFGS_Powell.cpp:70-192)
 *
 * Gate records are (type, target, control, param_start) with the ids of Gate.h:37-50.
 * Matrices are row-major interleaved complex128; the decomposer receives U^dagger.
 * Every function returns 0 on success, 1 for a gate list whose parameter layout differs
 * from the one the reference assigns, 2 when the reference threw.
 */
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "Gates_block.h"
#include "N_Qubit_Decomposition_custom.h"
#include "N_Qubit_Decomposition_Tree_Search.h"
#include "BFGS_Powell.h"
#include "config_element.h"

extern "C" void sqgr_blas_threads(int n);

namespace {

enum { kCZ = 4, kCNOT = 5, kU3 = 7, kRY = 8, kRX = 9, kRZ = 10, kCRY = 14 };

/* Builds the reference's Gates_block from the records; returns nullptr when a record's
 * param_start differs from the index the reference assigns (add order). */
Gates_block* build_block(int n, const int* g, int L) {
    Gates_block* b = new Gates_block(n);
    for (int i = 0; i < L; ++i) {
        const int type = g[4 * i], t = g[4 * i + 1], c = g[4 * i + 2];
        switch (type) {
            case kU3: b->add_u3(t); break;
            case kRX: b->add_rx(t); break;
            case kRY: b->add_ry(t); break;
            case kRZ: b->add_rz(t); break;
            case kCNOT: b->add_cnot(t, c); break;
            case kCZ: b->add_cz(t, c); break;
            case kCRY: b->add_cry(t, c); break;
            default: delete b; return nullptr;
        }
    }
    std::vector<Gate*> gates = b->get_gates();
    for (int i = 0; i < L; ++i) {
        if (gates[i]->get_parameter_num() > 0 && gates[i]->get_parameter_start_idx() != g[4 * i + 3]) {
            delete b;
            return nullptr;
        }
    }
    return b;
}

struct Problem {
    Gates_block* block = nullptr;
    N_Qubit_Decomposition_custom* dec = nullptr;
    ~Problem() {
        delete dec;
        delete block;
    }
};

/* N_Qubit_Decomposition_custom over a caller-owned U^dagger (rows x cols, no copy), with
 * the gate structure set as the wrapper's set_Gate_Structure does. */
bool make_problem(Problem& p, int n, const int* g, int L, double* udag, int cols, int trace_offset,
                  int variant) {
    p.block = build_block(n, g, L);
    if (p.block == nullptr) return false;
    Matrix U(reinterpret_cast<QGD_Complex16*>(udag), 1 << n, cols);
    std::map<std::string, Config_Element> config;
    p.dec = new N_Qubit_Decomposition_custom(U, n, false, config, RANDOM, 0);
    p.dec->set_verbose(0);
    p.dec->set_custom_gate_structure(p.block);
    p.dec->set_trace_offset(trace_offset);
    p.dec->set_cost_function_variant(static_cast<cost_function_type>(variant));
    return true;
}

long g_calls = 0;

void counted_combined(Matrix_real x, void* inst, double* f, Matrix_real& grad) {
    ++g_calls;
    Optimization_Interface::optimization_problem_combined(x, inst, f, grad);
}

}  // namespace

extern "C" {

void sqgr_init(void) { sqgr_blas_threads(1); }

int sqgr_cost(int n, const int* g, int L, const double* theta, int P, double* udag, int cols, int trace_offset,
              int variant, double* cost) {
    try {
        Problem p;
        if (!make_problem(p, n, g, L, udag, cols, trace_offset, variant)) return 1;
        Matrix_real x(const_cast<double*>(theta), 1, P);
        *cost = p.dec->optimization_problem(x);
        return 0;
    } catch (...) {
        return 2;
    }
}

int sqgr_cost_grad(int n, const int* g, int L, const double* theta, int P, double* udag, int cols,
                   int trace_offset, int variant, double* cost, double* grad) {
    try {
        Problem p;
        if (!make_problem(p, n, g, L, udag, cols, trace_offset, variant)) return 1;
        Matrix_real x(const_cast<double*>(theta), 1, P);
        Matrix_real gr(grad, P, 1);
        p.dec->optimization_problem_combined(x, cost, gr);
        return 0;
    } catch (...) {
        return 2;
    }
}

int sqgr_batch(int n, const int* g, int L, const double* theta, int P, int B, double* udag, int cols,
               int trace_offset, int variant, double* costs) {
    try {
        Problem p;
        if (!make_problem(p, n, g, L, udag, cols, trace_offset, variant)) return 1;
        std::vector<Matrix_real> rows(B);
        for (int b = 0; b < B; ++b) rows[b] = Matrix_real(const_cast<double*>(theta) + (size_t)b * P, 1, P);
        Matrix_real out = p.dec->optimization_problem_batched(rows);
        for (int b = 0; b < B; ++b) costs[b] = out[b];
        return 0;
    } catch (...) {
        return 2;
    }
}

int sqgr_apply_to(int n, const int* g, int L, const double* theta, int P, double* mtx, int rows, int cols,
                  int parallel) {
    try {
        Gates_block* b = build_block(n, g, L);
        if (b == nullptr) return 1;
        Matrix_real x(const_cast<double*>(theta), 1, P);
        Matrix m(reinterpret_cast<QGD_Complex16*>(mtx), rows, cols);
        b->apply_to(x, m, parallel);
        delete b;
        return 0;
    } catch (...) {
        return 2;
    }
}

int sqgr_apply_from_right(int n, const int* g, int L, const double* theta, int P, double* mtx, int rows,
                          int cols) {
    try {
        Gates_block* b = build_block(n, g, L);
        if (b == nullptr) return 1;
        Matrix_real x(const_cast<double*>(theta), 1, P);
        Matrix m(reinterpret_cast<QGD_Complex16*>(mtx), rows, cols);
        b->apply_from_right(x, m);
        delete b;
        return 0;
    } catch (...) {
        return 2;
    }
}

/* out receives the P derivative matrices, each rows x cols, back to back */
int sqgr_apply_derivate_to(int n, const int* g, int L, const double* theta, int P, const double* input, int rows,
                           int cols, int parallel, double* out) {
    try {
        Gates_block* b = build_block(n, g, L);
        if (b == nullptr) return 1;
        Matrix_real x(const_cast<double*>(theta), 1, P);
        Matrix in(reinterpret_cast<QGD_Complex16*>(const_cast<double*>(input)), rows, cols);
        std::vector<Matrix> d = b->apply_derivate_to(x, in, parallel);
        const size_t per = (size_t)rows * cols;
        for (size_t k = 0; k < d.size() && k < (size_t)P; ++k) {
            for (int r = 0; r < rows; ++r)
                std::memcpy(out + 2 * (k * per + (size_t)r * cols), d[k].get_data() + (size_t)r * d[k].stride,
                            sizeof(QGD_Complex16) * cols);
        }
        delete b;
        return d.size() == (size_t)P ? 0 : 2;
    } catch (...) {
        return 2;
    }
}

/* unitary (rows x cols) and the P derivative matrices of the circuit applied to U^dagger */
int sqgr_combined_unitary(int n, const int* g, int L, const double* theta, int P, double* udag, int cols,
                          double* unitary, double* derivs) {
    try {
        Problem p;
        if (!make_problem(p, n, g, L, udag, cols, 0, 0)) return 1;
        Matrix_real x(const_cast<double*>(theta), 1, P);
        Matrix U;
        std::vector<Matrix> dU;
        p.dec->optimization_problem_combined_unitary(x, U, dU);
        const int rows = 1 << n;
        for (int r = 0; r < rows; ++r)
            std::memcpy(unitary + 2 * (size_t)r * cols, U.get_data() + (size_t)r * U.stride, sizeof(QGD_Complex16) * cols);
        const size_t per = (size_t)rows * cols;
        for (size_t k = 0; k < dU.size() && k < (size_t)P; ++k)
            for (int r = 0; r < rows; ++r)
                std::memcpy(derivs + 2 * (k * per + (size_t)r * cols), dU[k].get_data() + (size_t)r * dU[k].stride,
                            sizeof(QGD_Complex16) * cols);
        return dU.size() == (size_t)P ? 0 : 2;
    } catch (...) {
        return 2;
    }
}

/* One BFGS_Powell run from x (updated in place) with at most max_iters iterations;
 * returns the final cost and the number of cost+gradient evaluations it made. */
int sqgr_bfgs_run(int n, const int* g, int L, int P, double* udag, int cols, int trace_offset, int variant,
                  double* x, long max_iters, double* cost, long* calls) {
    try {
        Problem p;
        if (!make_problem(p, n, g, L, udag, cols, trace_offset, variant)) return 1;
        Matrix_real xm(P, 1);
        std::memcpy(xm.get_data(), x, sizeof(double) * P);
        g_calls = 0;
        BFGS_Powell opt(counted_combined, p.dec);
        *cost = opt.Start_Optimization(xm, max_iters);
        *calls = g_calls;
        std::memcpy(x, xm.get_data(), sizeof(double) * P);
        return 0;
    } catch (...) {
        return 2;
    }
}

/* The reference's structure search on U^dagger (rows x rows) with all qubit pairs as the
 * topology; use_osr / use_graph_search select its modes (0/0 is the exhaustive level search).
 * Returns the CNOT count of the structure found and its decomposition error. */
int sqgr_tree_search(int n, double* udag, int use_osr, int use_graph_search, int level_max, double tolerance,
                     long long seed, int* cnots, double* error) {
  try {
    Matrix U(reinterpret_cast<QGD_Complex16*>(udag), 1 << n, 1 << n);
    std::map<std::string, Config_Element> config;
    auto put = [&](const char* key, long long v) {
      Config_Element e;
      e.set_property(key, v);
      config[key] = e;
    };
    put("use_osr", use_osr);
    put("use_graph_search", use_graph_search);
    put("tree_level_max", level_max);
    put("random_seed", seed);
    Config_Element tol;
    tol.set_property("optimization_tolerance", tolerance);
    config["optimization_tolerance"] = tol;
    N_Qubit_Decomposition_Tree_Search dec(U, n, config, 0);
    dec.set_verbose(0);
    dec.set_optimization_tolerance(tolerance);
    dec.start_decomposition();
    std::map<std::string, int> nums = dec.get_gate_nums();
    *cnots = nums.count("CNOT") ? nums["CNOT"] : 0;
    *error = dec.get_decomposition_error();
    return 0;
  } catch (...) {
    return 2;
  }
}

}  // extern "C"
