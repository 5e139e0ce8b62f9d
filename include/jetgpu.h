/*
 * jetgpu.h -- C-ABI of the GB300 (sm_103a) tensor-network contraction library.
 *
 * This is the drop-in boundary for Jet's contraction hot path. Every entry
 * point takes plain device pointers, sizes and a cudaStream_t passed as
 * `void *` (NULL = legacy default stream), returns an int status
 * (JETGPU_OK = 0) and records a message readable through jetgpu_last_error()
 * on failure. No entry point allocates device memory unless its comment says
 * so; scratch space is caller-owned ("workspace") and sized by the matching
 * *_workspace_size query. Tensors are row-major complex arrays: complex64 =
 * interleaved float (re, im), complex128 = interleaved double.
 *
 * Each declaration names the reference interface it replaces (paths relative
 * to the reference project root).
 */
#ifndef JETGPU_H
#define JETGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JETGPU_ABI_VERSION 1

/* Status codes. */
#define JETGPU_OK 0
#define JETGPU_ERR_INVALID 1     /* bad argument (shape, permutation, size) */
#define JETGPU_ERR_CUDA 2        /* a CUDA runtime/driver call failed */
#define JETGPU_ERR_UNSUPPORTED 3 /* valid request the library does not serve */
#define JETGPU_ERR_WORKSPACE 4   /* workspace missing or too small */
#define JETGPU_ERR_TIMEOUT 5     /* a bounded device wait gave up */
#define JETGPU_ERR_MEMORY 6      /* the device memory pool limit (jetgpu_set_pool_limit) */

/* Element types. */
#define JETGPU_C64 0  /* std::complex<float>  */
#define JETGPU_C128 1 /* std::complex<double> */

/* Arithmetic forms of a contraction. */
#define JETGPU_PREC_FP32 0   /* plain: complex FMA in the element type (FP32 or FP64) */
#define JETGPU_PREC_TF32X3 1 /* tcgen05 kind::tf32, hi/lo split, 3 products, FP32 accumulate */
#define JETGPU_PREC_AUTO 2   /* a split form (FP16x3 unless jetgpu_set_auto_form says otherwise)
                                where the shape suits the tensor cores, else plain */
#define JETGPU_PREC_BF16X3 3 /* tcgen05 kind::f16 on BF16 hi/lo splits, 3 products, FP32
                                accumulate: twice the TF32 rate, ~2^-17 truncation per product */
#define JETGPU_PREC_FP16X3 4 /* tcgen05 kind::f16 on FP16 hi/lo splits of power-of-two scaled
                                operands, 3 products, FP32 accumulate: twice the TF32 rate,
                                ~2^-22 truncation per product (TF32x3's) */
#define JETGPU_PREC_TUNED 5  /* per contraction key, the fastest of FP32, TF32X3 (either main
                                loop) and FP16X3 (either tile order), timed on first use
                                (jetgpu_autotune_*);
                                AUTO for small steps and for keys first met during capture */

/* Complex product algorithms for the tensor-core form. */
#define JETGPU_ALGO_4M 0 /* Cr = ArBr - AiBi, Ci = ArBi + AiBr */
#define JETGPU_ALGO_3M 1 /* P1 = ArBr, P2 = AiBi, P3 = (Ar+Ai)(Br+Bi): Cr = P1 - P2,
                            Ci = P3 - P1 - P2 (split forms only) */

/* ---------------------------------------------------------------------------
 * Memory, streams and graphs: the runtime under the C++ host API.
 * The reference allocates per operation (CudaTensor.hpp:158-160, 638-640);
 * here device memory comes from a caching allocator (freed blocks are kept
 * per size and reused, stream-ordered on the library stream) or from a
 * caller-sized arena for captured graphs.
 * ------------------------------------------------------------------------- */

/* Allocates `bytes` of device memory from the caching allocator (256-byte
 * aligned). Allocates device memory (cudaMalloc) only when no cached block
 * of the size class is free. */
int jetgpu_malloc(size_t bytes, void **ptr);

/* Returns a block from jetgpu_malloc to the cache. */
int jetgpu_free(void *ptr);

/* Releases every cached (free) block to the device. */
int jetgpu_release_cached(void);

/*
 * Caps the bytes jetgpu_malloc may hold at once (0: no cap, the default).
 * An allocation that would pass the cap fails with JETGPU_ERR_MEMORY before
 * any CUDA call, so running out of device memory can be injected on the host
 * (the C++ API turns it into a Jet::Exception). jetgpu_pool_bytes_in_use
 * reports the bytes jetgpu_malloc currently holds.
 */
int jetgpu_set_pool_limit(size_t bytes);
size_t jetgpu_pool_bytes_in_use(void);

/* NVTX ranges (nsys / ncu timelines) for host code above the C-ABI; the
 * library's own entry points mark themselves. No cost without a tool. */
void jetgpu_range_push(const char *name);
void jetgpu_range_pop(void);

/* Bytes currently handed out by / held in the caching allocator. */
int jetgpu_memory_stats(size_t *in_use, size_t *cached, size_t *peak_in_use);

/* The library's default stream for the host API (created on first use,
 * non-blocking with respect to the legacy stream). */
void *jetgpu_default_stream(void);

/* Copies: kind 0 host->device, 1 device->host, 2 device->device,
 * stream-ordered on `stream`. */
int jetgpu_memcpy(void *dst, const void *src, size_t bytes, int kind, void *stream);

/* Fills `bytes` of device memory with zero bytes (stream-ordered). */
int jetgpu_memset_zero(void *dst, size_t bytes, void *stream);

int jetgpu_stream_synchronize(void *stream);

/* Stream capture into an executable CUDA graph (cudaStreamBeginCapture /
 * EndCapture / GraphInstantiate), replay and destruction. */
int jetgpu_graph_begin(void *stream);
int jetgpu_graph_end(void *stream, void **graph_exec);
int jetgpu_graph_launch(void *graph_exec, void *stream);
int jetgpu_graph_destroy(void *graph_exec);

/* CUDA events for timing host loops above the boundary: create, record on a
 * stream, elapsed ms between two recorded events (waits for `end`), destroy. */
int jetgpu_event_create(void **event);
int jetgpu_event_record(void *event, void *stream);
int jetgpu_event_elapsed_ms(void *start, void *end, float *ms);
int jetgpu_event_destroy(void *event);

/* Message of the last failing call made by this host thread ("" if none). */
const char *jetgpu_last_error(void);

/* ABI version (JETGPU_ABI_VERSION) of the loaded library. */
int jetgpu_version(void);

/* Streaming multiprocessor count and compute capability of the current
 * device. */
int jetgpu_device_info(int *sm_count, int *cc_major, int *cc_minor);

/* Current device of the calling thread, and selection of it (the device
 * guard of CudaTensor<T, DEVICE>; reference CudaTensorHelpers.hpp:179-235).
 * Library streams and pools are per device. */
int jetgpu_get_device(int *device);
int jetgpu_set_device(int device);

/*
 * Index permutation, out-of-place.
 *   out[new multi-index] = in[old multi-index], new axis j = old axis perm[j].
 * shape: `rank` old dimensions (any sizes >= 1); perm: a permutation of
 * 0..rank-1. Bit-exact (a pure copy). Power-of-two tensors take a tiled
 * bit-permutation kernel; other shapes a mixed-radix gather kernel.
 * Replaces Permuter<QFlexPermuter|DefaultPermuter>::Transpose
 * (include/jet/permute/Permuter.hpp:49-119, QFlex.hpp:158-538,
 * Default.hpp:20-133) as used by Tensor::Transpose (Tensor.hpp:578-642).
 * `in` and `out` must not overlap.
 */
int jetgpu_permute(const void *in, void *out, int rank, const uint64_t *shape,
                   const int32_t *perm, int dtype, void *stream);

/*
 * Same permutation applied to `batch` tensors stored back to back
 * (in + b * size, out + b * size, size = prod(shape)).
 */
int jetgpu_permute_batched(const void *in, void *out, uint64_t batch, int rank,
                           const uint64_t *shape, const int32_t *perm,
                           int dtype, void *stream);

/*
 * Dense product of already-ordered operands, plain arithmetic:
 *   C[m x n] = A[m x k] * B[k x n], row-major, alpha = 1, beta = 0.
 * Covers all four cases of TensorHelpers::MultiplyTensorData
 * (include/jet/TensorHelpers.hpp:128-168: GEMM, GEMV, GEMV^T, DOTU; m or n
 * equal to 1 selects the vector kernels). Complex64 computes with FP32 FMA,
 * complex128 with FP64 FMA. k = 0 writes zeros.
 */
int jetgpu_multiply(const void *A, const void *B, void *C, uint64_t m,
                    uint64_t n, uint64_t k, int dtype, void *stream);

/*
 * Pairwise contraction with both transposes fused in:
 *   C[left ++ right] = sum_common A * B
 * a_perm orders A's axes as (left ++ common); b_perm orders B's axes as
 * (common ++ right); m, n, k are the products of the left, right and common
 * dimensions. Replaces Tensor::ContractTensors (include/jet/Tensor.hpp:708-752)
 * after its label algebra; the label algebra stays on the host.
 *
 * precision: JETGPU_PREC_FP32, JETGPU_PREC_TF32X3, JETGPU_PREC_BF16X3 or
 * JETGPU_PREC_FP16X3 (complex64 only; shapes with m or n below 2 take the
 * plain form), JETGPU_PREC_AUTO or JETGPU_PREC_TUNED. algo: JETGPU_ALGO_4M, or
 * JETGPU_ALGO_3M with TF32X3, BF16X3 or FP16X3 (three real products instead
 * of four; its workspace is jetgpu_contract_workspace_size_algo's). FP16X3 needs
 * |scale_a + scale_b| <= 126.
 * scale_a, scale_b: power-of-two exponents applied exactly to A and B before
 * the product (C = (2^scale_a A)(2^scale_b B)); 0 for none.
 * workspace: caller-owned device scratch of at least
 * jetgpu_contract_workspace_size(...) bytes (may be NULL when that is 0).
 * Products with one side at most 16 wide and k <= 64 (a gate on a large
 * tensor) read A and B in place through the permutations and need none.
 */
size_t jetgpu_contract_workspace_size(int a_rank, const uint64_t *a_shape,
                                      const int32_t *a_perm, int b_rank,
                                      const uint64_t *b_shape,
                                      const int32_t *b_perm, uint64_t m,
                                      uint64_t n, uint64_t k, int dtype,
                                      int precision);

int jetgpu_contract(const void *A, int a_rank, const uint64_t *a_shape,
                    const int32_t *a_perm, const void *B, int b_rank,
                    const uint64_t *b_shape, const int32_t *b_perm, void *C,
                    uint64_t m, uint64_t n, uint64_t k, int dtype,
                    int precision, int algo, int scale_a, int scale_b,
                    void *workspace, size_t workspace_bytes, void *stream);

/*
 * jetgpu_contract_workspace_size for a complex product algorithm: the 3M
 * split forms keep six planes per operand (the split adds hi, lo of re + im)
 * instead of four. The cblas_cgemm call this product stands in for is
 * TensorHelpers.hpp:47-61 (the reference has one complex algorithm).
 */
size_t jetgpu_contract_workspace_size_algo(int a_rank, const uint64_t *a_shape,
                                           const int32_t *a_perm, int b_rank,
                                           const uint64_t *b_shape, const int32_t *b_perm,
                                           uint64_t m, uint64_t n, uint64_t k, int dtype,
                                           int precision, int algo);

/*
 * Batched contraction: C[b] = contract(A[b], B[b]) for b < batch, C packed as
 * batch x m x n. a_batched / b_batched: 0, a shared operand (one tensor used
 * by every b); 1, `batch` tensors of the given shape back to back; 2, one
 * tensor whose permutation lists first the batch axes (extents multiplying to
 * `batch`, in batch-index order) and then the operand's own axes, so the
 * batch may sit anywhere in its layout and the product's permute pass moves
 * it (no separate reorder). Orderings, m, n, k, precision and scales as in
 * jetgpu_contract.
 * This is the slice batch of TensorNetwork::SliceIndices /
 * TaskBasedContractor (TensorNetwork.hpp:210-284, TaskBasedContractor.hpp:
 * 162-248): slice-dependent tensors carry the batch, slice-independent ones
 * are shared. A batched A with a shared B folds the batch into M (one product
 * of batch*m rows); otherwise the tensor-core and SIMT products run with a
 * batch grid dimension.
 */
size_t jetgpu_contract_batched_workspace_size(uint64_t batch, int a_rank,
                                              const uint64_t *a_shape,
                                              const int32_t *a_perm, int a_batched,
                                              int b_rank, const uint64_t *b_shape,
                                              const int32_t *b_perm, int b_batched,
                                              uint64_t m, uint64_t n, uint64_t k,
                                              int dtype, int precision);

int jetgpu_contract_batched(uint64_t batch, const void *A, int a_rank,
                            const uint64_t *a_shape, const int32_t *a_perm,
                            int a_batched, const void *B, int b_rank,
                            const uint64_t *b_shape, const int32_t *b_perm,
                            int b_batched, void *C, uint64_t m, uint64_t n,
                            uint64_t k, int dtype, int precision, int algo,
                            int scale_a, int scale_b, void *workspace,
                            size_t workspace_bytes, void *stream);

/*
 * jetgpu_contract_batched (no scales) passing operand exponents between the
 * steps of a path, so the FP16x3 form does not scan operands that an earlier
 * product wrote. a_emax / b_emax (device ints, may be NULL): the binary
 * exponent of the largest |re| or |im| of A / B as jetgpu_max_exponent
 * defines it, when known; values below -1000 mean not known, and the operand
 * is scanned. c_emax (device int, may be NULL): set, stream-ordered, to C's
 * exponent when the product runs on the tensor cores, and to a value below
 * -1000 otherwise. No counterpart in the reference.
 */
int jetgpu_contract_batched_hinted(uint64_t batch, const void *A, int a_rank,
                                   const uint64_t *a_shape, const int32_t *a_perm, int a_batched,
                                   const void *B, int b_rank, const uint64_t *b_shape,
                                   const int32_t *b_perm, int b_batched, void *C, uint64_t m,
                                   uint64_t n, uint64_t k, int dtype, int precision, int algo,
                                   const int *a_emax, const int *b_emax, int *c_emax,
                                   void *workspace, size_t workspace_bytes, void *stream);

/*
 * A group of small independent contractions in one launch (no counterpart in
 * the reference, which makes one BLAS call per step): task t computes
 * C_t[b] = A_t[b] B_t[b] for b < batch, C_t packed batch x m x n row-major,
 * in the plain form (complex FMA in the element type). Operands are read
 * through device offset tables: element (b, i, j) of A's m x k view is
 * A[a_bat[b] + a_row[i] + a_col[j]], of B's k x n view B[b_bat[b] + b_row[i]
 * + b_col[j]] (element offsets; a shared operand's bat table is zeros), so
 * any axis order and batch placement needs no transpose pass. `tasks` is a
 * device array of n_tasks (<= 256) descriptors; total_tiles is the sum over
 * the tasks of jetgpu_group_tiles(batch, m, n). No task may write another's
 * operands.
 */
typedef struct {
    const void *A;
    const void *B;
    void *C;
    uint64_t batch, m, n, k;
    const int64_t *a_bat, *a_row, *a_col;
    const int64_t *b_bat, *b_row, *b_col;
} jetgpu_group_task;

uint64_t jetgpu_group_tiles(uint64_t batch, uint64_t m, uint64_t n);
int jetgpu_contract_group(const jetgpu_group_task *tasks, int n_tasks, uint64_t total_tiles,
                          int dtype, void *stream);

/*
 * jetgpu_contract without a workspace argument and without allocating: for
 * callers that cannot allocate device memory when they contract -- inside a
 * CUDA stream capture, where cudaMalloc is illegal; under a host's own fixed
 * GPU memory budget (JNI/cgo services, embedded runtimes); in latency-bound
 * loops where cudaMalloc/cudaFree would synchronise the device. This entry
 * point has no counterpart in the reference.
 *
 * Scratch comes from one 32 MiB device array inside the library (every GPU
 * that loads the library holds it until the process exits); a contraction
 * whose jetgpu_contract_workspace_size exceeds
 * jetgpu_contract_noalloc_max_scratch() is rejected with
 * JETGPU_ERR_WORKSPACE. The first call on each device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture. All calls share the one array: calls
 * whose executions overlap on the GPU (different streams, or concurrent
 * graphs) race on it and must be serialised by the caller. The looked-up
 * address is cached per device for the life of the process: after a
 * cudaDeviceReset the module is loaded again and the array may move, so a
 * process that resets a device must not call this entry point on it again.
 * Arguments and results are those of jetgpu_contract.
 */
int jetgpu_contract_noalloc(const void *A, int a_rank, const uint64_t *a_shape,
                            const int32_t *a_perm, const void *B, int b_rank,
                            const uint64_t *b_shape, const int32_t *b_perm, void *C,
                            uint64_t m, uint64_t n, uint64_t k, int dtype,
                            int precision, int algo, int scale_a, int scale_b,
                            void *stream);

/* Bytes of scratch jetgpu_contract_noalloc can use (its size limit). */
size_t jetgpu_contract_noalloc_max_scratch(void);

/*
 * The two stages of the TF32x3 form of jetgpu_contract, for callers that
 * schedule them separately (batched executors, profilers).
 *
 * jetgpu_split_tf32: permutes a complex64 tensor (as jetgpu_permute) and
 * writes it, multiplied by 2^scale_exp, as fp32 planes holding TF32 values:
 * plane p at planes + p * plane_stride floats, p = 0 re_hi, 1 re_lo, 2 im_hi,
 * 3 im_lo (x = hi + lo + O(2^-22 |x|)) and, when n_planes == 6, 4 -im_hi,
 * 5 -im_lo; the permuted tensor is viewed as a rows x cols row-major matrix
 * stored with a row pitch of `pitch` floats (pitch >= cols, pitch % 4 == 0).
 *
 * jetgpu_gemm_tf32x3: C[m x n] (complex64, row-major) = A * B^T from the
 * planes of A (m x k, 4 planes) and B (n x k, i.e. B in (right ++ common)
 * order, jetgpu_tc_b_planes() planes), with row pitch kpitch; tcgen05
 * kind::tf32 tensor cores, three products per real product, FP32
 * accumulation, output multiplied by `out_scale`.
 * Replaces the cblas_cgemm call of TensorHelpers.hpp:47-61.
 *
 * jetgpu_set_tc_variant selects the main-loop shape of the tensor-core
 * products for the calling process: 0 = default (M 128 x N 128 MMAs over 4 B
 * planes, 3 stages of 64-byte rows); 1 = M 128 x N 256 MMAs over 6 B planes
 * (stacked [Br; Bi] and [-Bi; Br] operands, half the MMA count; TF32, BF16 and
 * FP16 through jetgpu_contract*); 2 = BF16 with 32-byte rows in 6 stages
 * (twice the pipeline depth in the same shared memory). jetgpu_tc_b_planes()
 * reports the B planes the TF32 stage product (jetgpu_gemm_tf32x3) reads; the
 * BF16 and FP16 stage products (jetgpu_gemm_bf16x3, jetgpu_gemm_fp16x3) always
 * read four.
 */
int jetgpu_split_tf32(const void *in, int rank, const uint64_t *shape,
                      const int32_t *perm, uint64_t rows, uint64_t cols,
                      uint64_t pitch, uint64_t plane_stride, int scale_exp,
                      int n_planes, float *planes, void *stream);

int jetgpu_set_tc_variant(int variant);
int jetgpu_tc_b_planes(void);

/*
 * jetgpu_set_tc_persistent(1) (the default) runs the tensor-core products as
 * one persistent CTA per SM walking the tiles, each tile's epilogue
 * overlapping the next tile's loads and MMAs; 0 launches one CTA per tile and
 * lets the hardware schedule them.
 */
int jetgpu_set_tc_persistent(int on);

/*
 * jetgpu_set_tc_group_m sets the tile order of the tensor-core products:
 * consecutive tiles walk `group_m` tile rows (128 rows each) down one tile
 * column before moving to the next column (default 8; 1 is row-major).
 */
int jetgpu_set_tc_group_m(int group_m);

/*
 * jetgpu_set_tc_chunk_depth sets, for the calling process, the K depth the
 * tensor-core products accumulate in tensor memory before folding the partial
 * sum into FP32 registers (round to nearest); 0 restores the defaults (16 for
 * TF32x3, 128 for BF16x3). The tensor core's own accumulation loses accuracy
 * with the depth it accumulates: shorter chunks are more accurate, longer
 * ones fold less often. Rounded down to whole stages (16 k for TF32, 32 for
 * BF16), at least one stage.
 */
int jetgpu_set_tc_chunk_depth(int k_depth);

/*
 * jetgpu_set_auto_form selects, for the calling process, the split form that
 * JETGPU_PREC_AUTO uses on the steps it gives to the tensor cores:
 * JETGPU_PREC_FP16X3 (the default), JETGPU_PREC_TF32X3 or JETGPU_PREC_BF16X3.
 */
int jetgpu_set_auto_form(int precision);

/*
 * The autotuner behind JETGPU_PREC_TUNED (no counterpart in the reference,
 * which has one BLAS form). The first contraction with a given key (device,
 * batch, batched operands, m, n, k, dtype, both shapes and permutations)
 * times each candidate form on the caller's stream after one untimed run and
 * keeps the fastest; later ones with that key run it directly, also inside a
 * stream capture. Steps whose m n k times the batch is below `mnk` (default
 * 2^20) take AUTO's rule. jetgpu_autotune_entry reports entry `index` (in the
 * order they were made): batch, m, n, k, the chosen precision, main-loop
 * variant and tile order (group_m, 0 = the jetgpu_set_tc_group_m setting),
 * and the measured ms per contraction of the JETGPU_AUTOTUNE_CANDIDATES
 * candidates: FP32, TF32X3 (variant 0), TF32X3 (variant 1), FP16X3, FP16X3
 * in row-major tile order (group_m 1), FP16X3 with the N = 256 main loop
 * (variant 1); -1: not timed.
 */
#define JETGPU_AUTOTUNE_CANDIDATES 6
int jetgpu_set_autotune_min_work(uint64_t mnk);
size_t jetgpu_autotune_count(void);
int jetgpu_autotune_entry(size_t index, uint64_t *batch_m_n_k, int *precision, int *variant,
                          int *group_m, float *times_ms);
int jetgpu_autotune_clear(void);

int jetgpu_gemm_tf32x3(const float *a_planes, const float *b_planes, void *C,
                       uint64_t m, uint64_t n, uint64_t k, uint64_t kpitch,
                       float out_scale, void *stream);

/*
 * The two stages of the BF16x3 form (JETGPU_PREC_BF16X3).
 *
 * jetgpu_split_bf16: as jetgpu_split_tf32 with 16-bit BF16 words: plane p
 * (0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo; hi = RN_bf16(x), lo = RN_bf16(x - hi),
 * x = hi + lo + O(2^-17 |x|)) at planes + p * plane_stride words, row pitch
 * `pitch` words (pitch >= cols, pitch % 8 == 0).
 *
 * jetgpu_gemm_bf16x3: C[m x n] = A * B^T from four BF16 planes of A (m x k)
 * and of B (n x k) with row pitch kpitch words; tcgen05 kind::f16 (BF16 in,
 * FP32 accumulate), three products per real product, output multiplied by
 * `out_scale`. Replaces the cblas_cgemm call of TensorHelpers.hpp:47-61.
 */
int jetgpu_split_bf16(const void *in, int rank, const uint64_t *shape,
                      const int32_t *perm, uint64_t rows, uint64_t cols,
                      uint64_t pitch, uint64_t plane_stride, int scale_exp,
                      uint16_t *planes, void *stream);

int jetgpu_gemm_bf16x3(const uint16_t *a_planes, const uint16_t *b_planes, void *C,
                       uint64_t m, uint64_t n, uint64_t k, uint64_t kpitch,
                       float out_scale, void *stream);

/*
 * The stages of the FP16x3 form (JETGPU_PREC_FP16X3), which keeps TF32x3's
 * precision (11 significant bits per piece) at the FP16 tensor rate. FP16's
 * range is covered by scaling each operand by 2^s before the split, s = 14 -
 * e_max clamped to [-120, 120], e_max from jetgpu_max_exponent on the device,
 * so the operand's largest magnitude lies in [2^14, 2^15).
 *
 * jetgpu_split_fp16: as jetgpu_split_bf16 with FP16 words of 2^s x
 * (hi = RN_fp16(2^s x), lo = RN_fp16(2^s x - hi)); *e_max_dev is read on the
 * device.
 *
 * jetgpu_gemm_fp16x3: C = A * B^T from four FP16 planes of A and of B;
 * e_max_dev points at two device ints, the max exponents of A and B, whose
 * scales the epilogue removes; the output is also multiplied by out_scale.
 */
int jetgpu_split_fp16(const void *in, int rank, const uint64_t *shape,
                      const int32_t *perm, uint64_t rows, uint64_t cols,
                      uint64_t pitch, uint64_t plane_stride, const int *e_max_dev,
                      uint16_t *planes, void *stream);

int jetgpu_gemm_fp16x3(const uint16_t *a_planes, const uint16_t *b_planes, void *C,
                       uint64_t m, uint64_t n, uint64_t k, uint64_t kpitch,
                       const int *e_max_dev, float out_scale, void *stream);

/*
 * The two stages of any split form, with either complex product algorithm.
 *
 * jetgpu_split_planes: fmt 0 TF32 (float words, pitch % 4 == 0), 1 BF16,
 * 2 FP16 (uint16 words, pitch % 8 == 0); planes 0-3 as above; extra 1 also
 * writes plane 4 = -im_hi and plane 5 = -im_lo (the B operand of the N = 256
 * main loop); extra 2 (JETGPU_ALGO_3M's operands) writes plane 4 = hi and
 * plane 5 = lo of re + im, and for FP16 scales by 2^(s - 1) instead of 2^s so
 * the sums stay below 2^15. extra 0 writes four planes. e_max_dev: FP16 only.
 *
 * jetgpu_gemm_split: C = A * B^T from the planes of A (m x k) and B (n x k):
 * algo JETGPU_ALGO_4M reads four planes of A and, with variant 0, four of B
 * (variant 1: the N = 256 main loop on six B planes written with extra 1);
 * JETGPU_ALGO_3M reads six per operand (written with extra 2) and forms
 * P1 = ArBr, P2 = AiBi, P3 = (Ar + Ai)(Br + Bi), Cr = P1 - P2,
 * Ci = P3 - P1 - P2 (variant ignored). e_max_dev: two device ints (A, B) for
 * FP16. Replaces the cblas_cgemm call of TensorHelpers.hpp:47-61.
 */
int jetgpu_split_planes(const void *in, int rank, const uint64_t *shape, const int32_t *perm,
                        uint64_t rows, uint64_t cols, uint64_t pitch, uint64_t plane_stride,
                        int fmt, int extra, const int *e_max_dev, void *planes, void *stream);

int jetgpu_gemm_split(const void *a_planes, const void *b_planes, void *C, uint64_t m,
                      uint64_t n, uint64_t k, uint64_t kpitch, int fmt, int algo, int variant,
                      const int *e_max_dev, float out_scale, void *stream);

/*
 * Element-wise sum C = A + B of equal-size tensors whose data are already in
 * the same index order (the transpose of B into A's order is a separate
 * jetgpu_permute). Replaces the data loop of Tensor::AddTensors
 * (include/jet/Tensor.hpp:446-451).
 */
int jetgpu_add(const void *A, const void *B, void *C, uint64_t size, int dtype,
               void *stream);

/* Element-wise complex conjugate (Tensor::Conj, Tensor.hpp:668-675). */
int jetgpu_conj(const void *in, void *out, uint64_t size, int dtype,
                void *stream);

/*
 * Cross-slice reduction in FP64: out[i] = sum_s results[s * size + i] for
 * s = 0..n_slices-1, summed in a fixed order in double precision; `out` is
 * complex128. Replaces the result reduction of
 * TaskBasedContractor::AddReductionTask (TaskBasedContractor.hpp:258-280),
 * which adds slice results with Tensor::AddTensors.
 * accumulate != 0 adds into the existing contents of `out`.
 */
int jetgpu_slice_sum_f64(const void *results, uint64_t n_slices, uint64_t size,
                         int dtype, void *out, int accumulate, void *stream);

/*
 * Device Tensor::SliceIndex for a run of slice values
 * (include/jet/Tensor.hpp:493-526 as driven by TensorNetwork::SliceIndices,
 * TensorNetwork.hpp:210-284). For s < n_values, with v = first_value + s,
 * axis axes[j] is fixed to (v / value_strides[j]) % shape[axes[j]] -- the
 * row-major unravel of the network-wide slice value v that SliceIndices
 * performs (Utilities.hpp:463-475) -- and out + s * out_size receives the
 * sub-tensor over the remaining axes in their original order
 * (out_size = product of the remaining dimensions).
 */
int jetgpu_slice_gather(const void *in, int rank, const uint64_t *shape,
                        int n_axes, const int32_t *axes,
                        const uint64_t *value_strides, uint64_t first_value,
                        uint64_t n_values, void *out, int dtype, void *stream);

/*
 * Adjoint of jetgpu_slice_gather for one slice value: full[positions of
 * slice `value`] += sliced, element for element (`sliced` holds out_size
 * elements in the order jetgpu_slice_gather writes them; `full` has `shape`).
 * The gradient of Tensor::SliceIndex (Tensor.hpp:493-526), used by the
 * adjoint of sliced network contractions. No counterpart in the reference.
 */
int jetgpu_slice_scatter_add(const void *sliced, int rank, const uint64_t *shape, int n_axes,
                             const int32_t *axes, const uint64_t *value_strides, uint64_t value,
                             void *full, int dtype, void *stream);

/*
 * jetgpu_slice_gather with the first slice value read from device memory
 * (*first_value_dev) when the kernel runs, so that one captured CUDA graph can
 * be replayed over successive chunks of slices; jetgpu_counter_add advances
 * such a device counter (*counter_dev += delta) in stream order.
 */
int jetgpu_slice_gather_at(const void *in, int rank, const uint64_t *shape,
                           int n_axes, const int32_t *axes,
                           const uint64_t *value_strides,
                           const uint64_t *first_value_dev, uint64_t n_values,
                           void *out, int dtype, void *stream);

int jetgpu_counter_add(uint64_t *counter_dev, uint64_t delta, void *stream);

/*
 * Reads and clears the device status word that bounded waits inside the
 * tensor-core kernels set on timeout (JETGPU_ERR_TIMEOUT), so that a hung
 * pipeline surfaces as an error on the host instead of a hang. Synchronous.
 */
int jetgpu_take_device_status(int *status);

/*
 * Exercises the failure path of the bounded device waits without faulting:
 * launches one kernel whose thread waits on an mbarrier that nothing
 * completes; the wait gives up after limit_us microseconds (1 us .. 1 s; or
 * 2^24 polls), records JETGPU_ERR_TIMEOUT in the status word that
 * jetgpu_take_device_status reads, and the kernel exits normally, so the
 * context stays usable. No reference counterpart (failure detection test).
 */
int jetgpu_probe_bounded_wait(unsigned int limit_us, void *stream);

/*
 * Largest binary exponent e with 2^e <= max |x_i| over the real and imaginary
 * parts of `size` complex elements, written to the device int *exp_dev
 * (stream-ordered, no host synchronisation). -1000 when every element is
 * zero. Used to choose the power-of-two scales of jetgpu_contract.
 */
int jetgpu_max_exponent(const void *x, uint64_t size, int dtype, int *exp_dev,
                        void *stream);

#ifdef __cplusplus
}
#endif

#endif /* JETGPU_H */
