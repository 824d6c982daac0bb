/* Testing aids of libaqsg: inspection of what the engine would run, for
 * host-side tests on machines without a GPU.  Not needed to use the engine.
 * Plain C, same conventions as aqsg.h (status codes, caller-owned buffers). */
#ifndef AQSG_DEBUG_H
#define AQSG_DEBUG_H

#include <stddef.h>
#include <stdint.h>

#include "aqsg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One tile pass of an encoded plan: tiles of 2^m amplitudes whose local
 * index bit i is global index bit tbits[i] (ascending; the L lowest are the
 * contiguous row bits), running table records [first, first + count).  A
 * tensor-core pass (tc = 1) keeps its fused unitaries' operands in the pool
 * at [tc_blob, tc_blob + tc_bytes); matk = 1: it also has dense k-qubit
 * ops for the CUDA cores. */
typedef struct aqsg_tile_pass {
    int32_t m, L, first, count;
    int32_t tbits[16];
    int32_t tc, matk;
    uint32_t tc_blob, tc_bytes;
} aqsg_tile_pass;

/* The tile-pass plan aqsg_apply_ops would run for ops in AQSG_EXEC_TILED mode
 * on an n-qubit register of dtype, after fusing at fuse_qubits (0: the gates
 * as they are), on a context whose aqsg_set_whole_tile_max setting is
 * whole_tile_max (0: the default) and aqsg_set_tensor_cores setting is
 * tensor_cores (2: the form the batched engine encodes, where fused
 * permutation matrices go to the tensor cores as well): the passes, the op
 * table (160-byte records: the engine's tile ops and register-phase ops) and
 * the operand pool, byte for byte as they are uploaded.  Call with NULL
 * buffers to get the counts and sizes. */
int aqsg_debug_tile_plan(int n, int dtype, const aqsg_op* ops, int count, int fuse_qubits,
                         int whole_tile_max, int tensor_cores, aqsg_tile_pass* passes, int pass_capacity,
                         int* pass_count,
                         void* table, size_t table_capacity, size_t* table_bytes,
                         void* pool, size_t pool_capacity, size_t* pool_bytes);

/* The plan image aqsg_batch_create uploads for a batch of circuits, byte
 * for byte: each size class's op table and operand pool, then the plans of
 * the registers of more than 14 qubits.  Built on the host, with the fusion
 * width fuse[k] and tensor-core choice tc[k] of the k-th register of more
 * than 14 qubits given instead of tuned (NULL: 0 for all).  With update
 * non-NULL: the image after aqsg_batch_update(update) instead.  Call with
 * image NULL to get the size. */
int aqsg_debug_batch_image(const aqsg_circuit* circuits, int count, const int* fuse, const int* tc,
                           const aqsg_circuit* update, void* image, size_t capacity, size_t* bytes);

/* Bytes the context currently holds in each of its scratch buffers, which
 * calls grow on demand with cudaMalloc: bytes[0..5] = FP64 partial sums,
 * sampling chunk prefixes, sampling uniforms, sampling outcomes, tile-pass
 * op tables, probability staging; *count = 6 (at most capacity written).
 * Tests use it to show that an entry point leaves these buffers alone. */
int aqsg_debug_ctx_scratch(aqsg_ctx ctx, size_t* bytes, int capacity, int* count);

#ifdef __cplusplus
}
#endif

#endif /* AQSG_DEBUG_H */
