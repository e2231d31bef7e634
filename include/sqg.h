/*
 * sqg.h — C ABI of the GB300 engine for SQUANDER's decomposition hot path:
 * the cost and gradient of a parametric gate circuit applied to a 2^n x cols
 * complex128 target (SQUANDER hands the decomposer U^dagger and minimises
 * f = 1 - Re Tr(C(theta) U^dagger)/cols by default).
 *
 * Conventions (identical to SQUANDER):
 *   - matrices are row-major interleaved complex128 {re, im}; row stride and batch
 *     stride are counted in complex elements; rows = 2^qbit_num;
 *   - qubit q is bit q of the row index (LSB = qubit 0);
 *   - gates[0] is applied first: C = G_{L-1} ... G_0;
 *   - parameters are contiguous in gate order; U3 stores (theta/2, phi, lambda),
 *     RX/RY/RZ/CRY store theta/2; kernels use sin/cos of the stored value.
 *
 * Every pointer argument named *_dev is device memory owned by the caller; apart from
 * the gate table that sqg_circuit_create copies to the device, the engine allocates no
 * device memory.  Calls are asynchronous on the given CUDA stream
 * (cudaStream_t passed as void*, NULL = legacy default stream) and return a status
 * code; no C++ exception crosses this boundary.  A circuit handle is immutable after
 * creation (apart from sqg_circuit_set_partitions, which replaces its state-vector plan)
 * and may be used from several threads and streams at once.
 */
#ifndef SQG_H
#define SQG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define SQG_OK 0
#define SQG_ERR_INVALID_ARGUMENT 1
#define SQG_ERR_UNSUPPORTED 2
#define SQG_ERR_WORKSPACE 3
#define SQG_ERR_CUDA 4
#define SQG_ERR_PARAMETER_COUNT 5

/* Gate type ids, equal to SQUANDER's gate_type enum (src-cpp/gates/include/Gate.h:37-50). */
#define SQG_CZ 4
#define SQG_CNOT 5
#define SQG_U3 7
#define SQG_RY 8
#define SQG_RX 9
#define SQG_RZ 10
#define SQG_CRY 14

/* Cost-function variants, equal to SQUANDER's cost_function_type
 * (src-cpp/decomposition/include/Optimization_Interface.h:43-45). */
#define SQG_FROBENIUS_NORM 0
#define SQG_HILBERT_SCHMIDT_TEST 3
#define SQG_INFIDELITY 9

/* One gate.  control = -1 for uncontrolled gates.  param_start is the index of the
 * gate's first parameter in the parameter vector (Gates_block::add_gate,
 * src-cpp/gates/Gates_block.cpp:2500-2525). */
typedef struct sqg_gate {
  int32_t type;
  int32_t target;
  int32_t control;
  int32_t param_start;
} sqg_gate;

typedef struct sqg_circuit sqg_circuit;

/* Human-readable text of a status code, or of the last error on this thread. */
const char* sqg_status_string(int status);
const char* sqg_last_error(void);

/* Builds a circuit handle from a flat gate list (nested SQUANDER blocks are flattened
 * by the caller in order).  Replaces the gate structure a decomposition receives via
 * set_Gate_Structure (squander/decomposition/qgd_N_Qubit_Decompositions_Wrapper.cpp:899)
 * and the gate list of Gates_block (src-cpp/gates/Gates_block.cpp:2500).  qbit_num
 * 1..30; the matrix entry points (cost, gradient, application to matrices, combined
 * unitary, ragged batches) accept up to 13 qubits, the batched decompositions up to 5, the
 * state-vector application up to 30.  Copies the gate table and the fused state-vector
 * plan to the current device. */
int sqg_circuit_create(int qbit_num, const sqg_gate* gates, int gate_num, sqg_circuit** out);
int sqg_circuit_destroy(sqg_circuit* circuit);
int sqg_circuit_param_num(const sqg_circuit* circuit);
int sqg_circuit_qbit_num(const sqg_circuit* circuit);
int sqg_circuit_gate_num(const sqg_circuit* circuit);

/* Workspace bytes needed by sqg_cost_grad for this circuit, batch and target width. */
size_t sqg_cost_grad_workspace_bytes(const sqg_circuit* circuit, int batch, int cols, int with_grad);

/* Cost and (optionally) gradient of `batch` parameter vectors.
 *   theta_dev   batch x P doubles (row stride P);
 *   target_dev  rows x cols complex128 (U^dagger), shared by all instances when
 *               target_batch_stride == 0, else one per instance at that stride;
 *   cost_dev    batch doubles;  grad_dev  batch x P doubles or NULL (cost only).
 * Replaces Optimization_Interface::optimization_problem (Optimization_Interface.cpp:634-668),
 * optimization_problem_batched (:940-1033) and optimization_problem_combined_non_static
 * (:1145-1485) of the CPU reference, for the cost variants listed above.  The gradient
 * is the adjoint (reverse-sweep) gradient; checkpoint_interval > 0 stores the forward
 * state every that many gates in the workspace and restores it during the reverse sweep
 * instead of relying on uncomputation alone (0 = pure uncomputation). */
int sqg_cost_grad(const sqg_circuit* circuit, const double* theta_dev, int batch, const void* target_dev, int cols,
                  long long target_batch_stride, int trace_offset, int cost_variant, double* cost_dev,
                  double* grad_dev, int checkpoint_interval, void* workspace_dev, size_t workspace_bytes,
                  void* stream);
size_t sqg_cost_grad_checkpoint_workspace_bytes(const sqg_circuit* circuit, int batch, int cols,
                                                int checkpoint_interval);

/* Size of the scratch array built into the library for sqg_cost_grad_noalloc (32 MiB). */
#define SQG_NOALLOC_SCRATCH_BYTES (32u << 20)

/* sqg_cost_grad for callers that cannot allocate device memory.  No counterpart in the
 * reference: it exists for callers such as a cost callback plugged into an optimizer
 * interface that hands over only the parameters, the cost and the gradient (there is no
 * place to pass a workspace and the callback runs thousands of times), or code whose
 * device memory belongs to a framework allocator that forbids raw cudaMalloc.  Same
 * arguments, checks and results as sqg_cost_grad minus the workspace: the scratch is a
 * 32 MiB array compiled into the library, which every GPU that loads the library holds until
 * the process exits.  Requests needing more scratch than SQG_NOALLOC_SCRATCH_BYTES (see
 * sqg_cost_grad_workspace_bytes) fail with SQG_ERR_WORKSPACE; gradients up to five qubits
 * without checkpoints need none.  The first call in each CUDA context (normally once per
 * device) looks up the array's device address with cudaGetSymbolAddress in that context;
 * make that first call before any stream capture (after a cudaDeviceReset the device has a
 * new context and the next call does the set-up again).  All calls share the one array, so
 * calls that overlap on the GPU (other streams, other host threads) race; the array keeps the
 * last call's contents and every byte a call reads is written earlier in the same call.
 * Allocates nothing. */
int sqg_cost_grad_noalloc(const sqg_circuit* circuit, const double* theta_dev, int batch, const void* target_dev,
                          int cols, long long target_batch_stride, int trace_offset, int cost_variant,
                          double* cost_dev, double* grad_dev, int checkpoint_interval, void* stream);

/* ---- Ragged batches: instances with different circuits (qubit counts) in one launch ----
 * Plans the evaluation of `count` instances, instance i with circuits[i] (its own qubit
 * count, gates and parameters) against its own 2^n_i x cols[i] target.  Parameters,
 * targets and gradients are packed flat in instance order; sqg_ragged_layout returns the
 * count+1 offsets (in doubles for parameters/gradients, complex elements for targets).
 * tile_cols (optional, per instance, 0 = automatic) fixes the column-tile width, for
 * autotuning.  The launch is a persistent grid pulling (instance, tile) work items from a
 * queue ordered by decreasing work; kernel attributes are set at planning time, so the
 * calls of sqg_ragged_cost_grad can be captured in a CUDA graph.  Replaces the reference's
 * per-instance loop of Optimization_Interface::optimization_problem_batched
 * (Optimization_Interface.cpp:940-1033), which requires one shared circuit. */
typedef struct sqg_ragged_batch sqg_ragged_batch;
int sqg_ragged_create(const sqg_circuit* const* circuits, const int* cols, int count, int with_grad,
                      const int* tile_cols, sqg_ragged_batch** out);
int sqg_ragged_destroy(sqg_ragged_batch* batch);
size_t sqg_ragged_workspace_bytes(const sqg_ragged_batch* batch);
int sqg_ragged_layout(const sqg_ragged_batch* batch, long long* theta_offsets, long long* target_offsets);
int sqg_ragged_cost_grad(const sqg_ragged_batch* batch, const double* theta_dev, const void* targets_dev,
                         int cost_variant, double* cost_dev, double* grad_dev, void* workspace_dev,
                         size_t workspace_bytes, void* stream);

/* Workspace bytes needed by sqg_apply. */
size_t sqg_apply_workspace_bytes(const sqg_circuit* circuit, int batch);

/* In-place left application M_b <- C(theta_b) M_b for `batch` matrices of rows x cols
 * (row stride `stride`, batch stride `batch_stride`, both in complex elements).
 * fused = 1: every gate applied to shared-memory column tiles in one pass over the
 * matrix; fused = 0: one pass over the matrix per gate.  Replaces Gates_block::apply_to
 * (src-cpp/gates/Gates_block.cpp:606-710) and Circuit.apply_to
 * (squander/gates/qgd_Circuit.py:546). */
int sqg_apply(const sqg_circuit* circuit, const double* theta_dev, int batch, void* mtx_dev, int cols,
              long long stride, long long batch_stride, int fused, void* workspace_dev, size_t workspace_bytes,
              void* stream);

/* In-place right application M <- M C(theta) (cols = 2^qbit_num).  Replaces
 * Gates_block::apply_from_right (src-cpp/gates/Gates_block.cpp:885-935). */
/* State vectors (cols = 1) of up to 30 qubits: applies the circuit in place to batch
 * vectors of 2^qbit_num amplitudes (vector b at states_dev + b * state_stride, stride >=
 * 2^qbit_num).  Replaces Gate::apply_to / Gates_block::apply_to on state-vector inputs
 * (src-cpp/gates/Gate.cpp:1710-1726, apply_kernel_to_state_vector_input*; driven by
 * examples/simulation/QC_sim_benchmark.py).  fused != 0 groups consecutive gates whose qubits,
 * together with the five lowest, number at most 12 into blocks (the role of the reference's
 * partitioning into fused blocks, squander/partitioning) and applies each block to chunks of
 * 4096 amplitudes in shared memory: one read and write of the state per block
 * (sqg_state_block_count); fused == 0 makes one pass per gate.  Circuit handles of more than
 * 13 qubits are accepted only by this entry point.  Workspace: sqg_state_workspace_bytes. */
size_t sqg_state_workspace_bytes(const sqg_circuit* circuit, int batch);
int sqg_state_block_count(const sqg_circuit* circuit);

/* Hands a partitioning of the gate list to the fused state-vector plan: part_ends[i] is the
 * gate index after partition i (non-decreasing, the last equal to gate_num).  Fused passes
 * then start only at partition boundaries, consecutive partitions merged while their qubits
 * with the five lowest number at most 12 (a partition larger than that is split gate by gate);
 * nparts == 0 restores the gate-by-gate plan.  The partitions come from the partitioner
 * (squander/partitioning/partition.py:PartitionCircuit, kahn.py), which reorders the gates so
 * that each partition spans few qubits.  Rebuilds the plan synchronously; no work that uses
 * the circuit may be in flight. */
int sqg_circuit_set_partitions(sqg_circuit* circuit, const int* part_ends, int nparts);
int sqg_apply_state(const sqg_circuit* circuit, const double* theta_dev, int batch, void* states_dev,
                    long long state_stride, int fused, void* workspace_dev, size_t workspace_bytes, void* stream);

int sqg_apply_from_right(const sqg_circuit* circuit, const double* theta_dev, void* mtx_dev, int rows,
                         long long stride, void* workspace_dev, size_t workspace_bytes, void* stream);

/* Forward matrix and all P derivative matrices: out_dev holds P+1 matrices of
 * rows x cols (dense, stride cols): out[0] = C(theta) target, out[1+k] = dC/dtheta_k target.
 * Replaces Optimization_Interface::optimization_problem_combined_unitary
 * (Optimization_Interface.cpp:1525-1547) and Gates_block::apply_to_combined / apply_derivate_to
 * (src-cpp/gates/Gates_block.cpp:1012-1150, 1328-1364). */
int sqg_combined_unitary(const sqg_circuit* circuit, const double* theta_dev, const void* target_dev, int cols,
                         void* out_dev, void* workspace_dev, size_t workspace_bytes, void* stream);

/* Batched decomposition of `batch` small targets (qbit_num <= 6, the instance's shared memory
 * within the device's per-CTA limit), one complete BFGS decomposition per CTA, entirely on
 * the device.
 *   targets_dev  batch x rows x cols complex128 (each U^dagger);
 *   x_dev        batch x P doubles: start points in, best parameters out;
 *   cost_dev     batch doubles out (best cost);  calls_dev  batch ints out (cost+gradient
 *                evaluations used);  iters_dev  batch ints out (BFGS iterations) or NULL.
 * Each instance runs up to max_outer outer iterations of iteration_loops BFGS runs of at
 * most max_calls evaluations, perturbing the best point by U[0, 2 pi)/100 after an
 * improvement, and stops once the best cost is below `tolerance`; with
 * stop_at_tolerance != 0 a run also stops at the first evaluation below it.  Replaces
 * N_Qubit_Decomposition_custom::start_decomposition with the BFGS optimizer
 * (src-cpp/decomposition/N_Qubit_Decomposition_custom.cpp:116-190,
 * src-cpp/optimization_engines/BFGS.cpp:42-152, src-cpp/common/BFGS_Powell.cpp:70-396).
 * The workspace holds the per-instance BFGS matrices when they do not fit on chip. */
size_t sqg_decompose_workspace_bytes(const sqg_circuit* circuit, int batch, int cols);
int sqg_decompose_batched(const sqg_circuit* circuit, const void* targets_dev, int cols, int batch, int trace_offset,
                          int cost_variant, double* x_dev, double* cost_dev, int* calls_dev, int* iters_dev,
                          double tolerance,
                          int max_calls, int max_outer, int iteration_loops, int stop_at_tolerance,
                          unsigned long long seed, void* workspace_dev, size_t workspace_bytes, void* stream);

/* One BFGS decomposition for any qbit_num the gradient supports (<= 12), run on the device as
 * a single CUDA graph launch: a conditional while-node whose body evaluates the cost and
 * gradient (the kernels of sqg_cost_grad) and then advances BFGS_Powell (Powell's Z update, the
 * reference line search, the restarts) on one CTA up to the next point to evaluate.  Replaces
 * the host loop of solve_layer_optimization_problem_BFGS (src-cpp/optimization_engines/
 * BFGS.cpp:42-152, src-cpp/common/BFGS_Powell.cpp:70-396).  Semantics and parameters as
 * sqg_decompose_batched with batch 1 (same random stream for the restart perturbations); up to
 * five qubits and for targets with cols >= 3N/4 the result is bit-identical to
 * sqg_decompose_batched.  The workspace (256-byte aligned, sqg_bfgs_loop_workspace_bytes) holds
 * the state, the P x P matrix Z and the evaluation scratch and must stay untouched until the
 * stream reaches the end of the call.  Asynchronous on stream. */
size_t sqg_bfgs_loop_workspace_bytes(const sqg_circuit* circuit, int cols);
int sqg_decompose_bfgs_loop(const sqg_circuit* circuit, const void* target_dev, int cols, int trace_offset,
                            int cost_variant, double* x_dev, double* cost_dev, int* calls_dev, int* iters_dev,
                            double tolerance, int max_calls, int max_outer, int iteration_loops,
                            int stop_at_tolerance, unsigned long long seed, void* workspace_dev,
                            size_t workspace_bytes, void* stream);

/* Batched BFGS decompositions of many gate STRUCTURES at once (the inner loop of the
 * structure-search decomposers, N_Qubit_Decomposition_Tree_Search::
 * tree_search_over_gate_structures, src-cpp/decomposition/N_Qubit_Decomposition_Tree_Search.cpp:
 * 1269-1451, which runs one N_Qubit_Decomposition_custom per candidate structure): instance b
 * decomposes with its own gate list gates[b * gate_num .. (b + 1) * gate_num) (HOST array of
 * batch x gate_num records).  Every list repeats the gate types and parameter layout of
 * `circuit`; only target and control qubits may differ (checked, then copied to the
 * workspace).  targets_dev + b * target_stride is instance b's target (target_stride 0: one
 * shared target).  Otherwise as sqg_decompose_batched.  Workspace (256-byte aligned):
 * sqg_decompose_structures_workspace_bytes. */
size_t sqg_decompose_structures_workspace_bytes(const sqg_circuit* circuit, int batch, int cols);
int sqg_decompose_structures(const sqg_circuit* circuit, const sqg_gate* gates, const void* targets_dev,
                             long long target_stride, int cols, int batch, int trace_offset, int cost_variant,
                             double* x_dev, double* cost_dev, int* calls_dev, int* iters_dev, double tolerance,
                             int max_calls, int max_outer, int iteration_loops, int stop_at_tolerance,
                             unsigned long long seed, void* workspace_dev, size_t workspace_bytes, void* stream);

/* Batched decompositions with SQUANDER's ADAM engine: replaces
 * Optimization_Interface::solve_layer_optimization_problem_ADAM
 * (src-cpp/optimization_engines/ADAM.cpp:44-330) with its Adam optimizer
 * (src-cpp/common/Adam.cpp: beta1 0.68, beta2 0.8, epsilon 1e-4, local-minimum test) and
 * randomize_parameters (src-cpp/decomposition/Optimization_Interface.cpp:576-607), the
 * optimizer N_Qubit_Decomposition_custom selects above five qubits
 * (N_Qubit_Decomposition_custom.cpp:59-76), here for qbit_num <= 6 with one CTA per target.
 * Each target runs up to max_outer engine calls of at most max_iters cost+gradient
 * evaluations (learning rate eta, adaptive as in the reference when adaptive_eta != 0, at
 * most random_shift_count_max randomisations, randomisation after randomization_threshold
 * evaluations without progress); it stops once the cost is below tolerance.  x (batch x P)
 * holds the start points on entry and the best points on exit; cost receives the minimum,
 * evals the evaluation count and shifts (nullable) the number of randomisations.  Random
 * numbers come from a splitmix64 stream seeded with seed + 7919 b for target b.  Needs no
 * workspace; asynchronous on stream. */
int sqg_decompose_batched_adam(const sqg_circuit* circuit, const void* targets_dev, int cols, int batch,
                               int trace_offset, int cost_variant, double* x_dev, double* cost_dev, int* evals_dev,
                               int* shifts_dev, double tolerance, int max_iters, double eta, int adaptive_eta,
                               int random_shift_count_max, long long randomization_threshold, int max_outer,
                               unsigned long long seed, void* stream);

/* Batched ADAM decompositions of many gate STRUCTURES at once: sqg_decompose_structures with
 * the engine of sqg_decompose_batched_adam, the optimizer the structure-search decomposers use
 * above five qubits (N_Qubit_Decomposition_Tree_Search.cpp:1487-1495 sets ADAM with
 * max_inner_iterations P / 852 * 1e7 and random_shift_count_max 5 for each candidate's
 * N_Qubit_Decomposition_custom).  Instance b decomposes with gate list gates[b * gate_num ..),
 * checked against `circuit` as in sqg_decompose_structures, target targets_dev + b *
 * target_stride (0: one shared target), random numbers seeded with seed + 7919 b; otherwise as
 * sqg_decompose_batched_adam.  The workspace (256-byte aligned,
 * sqg_decompose_structures_adam_workspace_bytes) holds the staged gate lists. */
size_t sqg_decompose_structures_adam_workspace_bytes(const sqg_circuit* circuit, int batch);
int sqg_decompose_structures_adam(const sqg_circuit* circuit, const sqg_gate* gates, const void* targets_dev,
                                  long long target_stride, int cols, int batch, int trace_offset, int cost_variant,
                                  double* x_dev, double* cost_dev, int* evals_dev, int* shifts_dev, double tolerance,
                                  int max_iters, double eta, int adaptive_eta, int random_shift_count_max,
                                  long long randomization_threshold, int max_outer, unsigned long long seed,
                                  void* workspace_dev, size_t workspace_bytes, void* stream);

/* One decomposition with SQUANDER's ADAM engine for any qbit_num the gradient supports
 * (<= 12), run on the device as a single CUDA graph launch: a conditional while-node whose
 * body evaluates the cost and gradient (the kernels of sqg_cost_grad) and then takes one
 * pass of the engine loop on one CTA, with no host round trip between evaluations.  Replaces
 * the host loop of Optimization_Interface::solve_layer_optimization_problem_ADAM
 * (src-cpp/optimization_engines/ADAM.cpp:44-330), the optimizer
 * N_Qubit_Decomposition_custom selects above five qubits (N_Qubit_Decomposition_custom.cpp:
 * 59-76).  The engine's semantics and parameters are those of sqg_decompose_batched_adam
 * with batch 1; current_minimum is the running minimum the first engine call starts with
 * (Decomposition_Base's current_minimum; DBL_MAX for a fresh decomposition), and the random
 * numbers come from a splitmix64 stream seeded with seed.  target_dev is N x cols (U dagger),
 * x_dev (P) holds the start point on entry and the best point on exit; cost_dev, evals_dev
 * and shifts_dev (nullable) are single values.  The workspace (256-byte aligned,
 * sqg_adam_loop_workspace_bytes) holds the engine state and the evaluation scratch and must
 * stay untouched until the stream reaches the end of the call.  Asynchronous on stream. */
size_t sqg_adam_loop_workspace_bytes(const sqg_circuit* circuit, int cols);
int sqg_decompose_adam_loop(const sqg_circuit* circuit, const void* target_dev, int cols, int trace_offset,
                            int cost_variant, double* x_dev, double* cost_dev, int* evals_dev, int* shifts_dev,
                            double tolerance, int max_iters, double eta, int adaptive_eta,
                            int random_shift_count_max, long long randomization_threshold, int max_outer,
                            double current_minimum, unsigned long long seed, void* workspace_dev,
                            size_t workspace_bytes, void* stream);

/* Measures the FP64 FMA peak of the current device in TFLOP/s (an FMA counts 2 flops) with
 * independent DFMA chains on 8 CTAs per SM, timed with CUDA events; scratch_dev receives
 * the chains' results (sqg_probe_fp64_scratch_bytes() bytes).  With active_lanes < 32 only
 * that many lanes of each warp compute while the rate is still reported for full warps,
 * which shows how the FP64 pipe charges partially active warps.  The roofline denominator
 * of the FP64-bound kernels.  No counterpart in the reference (measurement utility). */
size_t sqg_probe_fp64_scratch_bytes(void);
int sqg_probe_fp64_tflops(double* tflops, int active_lanes, void* scratch_dev, size_t scratch_bytes, void* stream);

/* ---- Learned initialiser kernels (BF16 operands, FP32 accumulation) --------------------
 * The initialiser maps a target to starting angles; it has no counterpart in the reference
 * (SQUANDER starts from zeros, random or close-to-zero angles, Decomposition_Base.cpp:415-436),
 * and only proposes start points to the decomposition kernels.  All pointers are device
 * pointers; bf16 buffers are `void*` holding IEEE bfloat16. */
/* C[M][N] = sum_k A'[m][k] B'[k][n] (+ bias[n]) (ReLU if relu) (+ C if accumulate), written as
 * fp32 to C and/or bf16 to C_bf16 (row stride N both).  A' = A (M x K, row stride lda) or A^T
 * (A stored K x M) when transA; B' = B (K x N, row stride ldb) or B^T (B stored N x K). */
int sqg_mlp_gemm_bf16(int M, int N, int K, const void* A, int lda, int transA, const void* B, int ldb, int transB,
                      float* C, int ldc, const float* bias, int relu, void* C_bf16, int accumulate, void* stream);
int sqg_mlp_to_bf16(const float* x, void* y_bf16, long long n, void* stream);
/* dA <- dA * (Z > 0) in place, with a bf16 copy. */
int sqg_mlp_relu_backward(float* dA, const float* Z, void* dZ_bf16, long long n, void* stream);
/* db[n] = sum_m dZ[m][n]. */
int sqg_mlp_col_sum(const float* dZ, int M, int N, float* db, void* stream);
/* Adam step (bias-corrected, step >= 1) on fp32 weights; refreshes w_bf16 when non-null. */
int sqg_mlp_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, float lr, float beta1,
                 float beta2, float eps, int step, float weight_decay, void* stream);
/* Angle head: out is M x 2P (cos, sin) pairs; theta = atan2.  mode 0: angles only; mode 1:
 * supervised loss against target angles (loss_rows, out_grad); mode 2: out_grad = chain
 * rule of dL/dtheta through atan2.  Gradients are multiplied by scale. */
int sqg_mlp_angle_head(const float* out, int M, int P, double* theta, const double* target_or_dtheta, int mode,
                       float scale, float* out_grad, float* loss_rows, void* stream);
/* Network input: interleaved Re/Im of n_complex complex128 values as bf16. */
int sqg_mlp_features(const void* U, long long n_complex, void* x_bf16, void* stream);
/* C[M][N] = A[M][K] B[N][K]^T (+ bias, ReLU) on the tcgen05 tensor cores (accumulator in
 * TMEM, operands staged by TMA with 128-byte swizzle); A and B bf16 row-major (K-major),
 * K, lda, ldb multiples of 8, 16-byte aligned.  Waits inside the kernel are bounded: a
 * time-out writes a non-zero code to *err_dev (device int) instead of hanging. */
int sqg_mlp_gemm_tc(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* C, int ldc,
                    const float* bias, int relu, void* C_bf16, int* err_dev, void* stream);
/* out[c][r] = in[r][c] for a rows x cols bf16 matrix. */
int sqg_mlp_transpose_bf16(const void* in, int rows, int cols, int ld_in, void* out, int ld_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SQG_H */
