/*
 * C restatement of the reference Jet CPU permuters.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle and the timed CPU baseline ("port") of
 * bench.py. Nothing in jet_gb300/ links or loads this file.
 *
 * oracle_permute restates DefaultPermuter::Transpose
 * (include/jet/permute/Default.hpp:20-133): the old linear index is walked in
 * blocks of BLOCKSIZE = 1024 positions; for each block an odometer over the
 * old multi-index produces the new position of every element, then the block
 * is scattered. Two differences, both deliberate:
 *   - new positions are kept in 64 bits (the reference stores them in
 *     `unsigned short`, Default.hpp:85-86, which wraps beyond 65536 elements);
 *   - blocks run in parallel with OpenMP, as the reference's QFlex passes do
 *     (QFlex.hpp:172-217), so the CPU baseline uses every host core.
 * Elements are copied as opaque `elem_bytes`-sized records, so the result is
 * bit-exact for any element type.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_BLOCK 1024
#define ORACLE_MAX_RANK 64

int oracle_permute(const void *in, void *out, int rank, const uint64_t *shape,
                   const int32_t *perm, int elem_bytes, int nthreads)
{
    if (rank < 0 || rank > ORACLE_MAX_RANK || elem_bytes <= 0)
        return 1;
    uint64_t total = 1;
    for (int i = 0; i < rank; ++i)
        total *= shape[i];
    if (total == 0)
        return 0;
    /* map_old_to_new_idxpos and the super-dimensions (Default.hpp:37-59). */
    int new_pos_of_old[ORACLE_MAX_RANK];
    uint64_t new_dims[ORACLE_MAX_RANK], old_super[ORACLE_MAX_RANK], new_super[ORACLE_MAX_RANK];
    for (int j = 0; j < rank; ++j) {
        if (perm[j] < 0 || perm[j] >= rank)
            return 1;
        new_pos_of_old[perm[j]] = j;
        new_dims[j] = shape[perm[j]];
    }
    if (rank > 0) {
        old_super[rank - 1] = 1;
        new_super[rank - 1] = 1;
        for (int i = rank - 1; i > 0; --i) {
            old_super[i - 1] = old_super[i] * shape[i];
            new_super[i - 1] = new_super[i] * new_dims[i];
        }
    }
    /* Stride in the output of a unit step of old axis i. */
    uint64_t step[ORACLE_MAX_RANK];
    for (int i = 0; i < rank; ++i)
        step[i] = new_super[new_pos_of_old[i]];
    const uint64_t nblocks = (total + ORACLE_BLOCK - 1) / ORACLE_BLOCK;
    const char *src = (const char *)in;
    char *dst = (char *)out;
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (uint64_t b = 0; b < nblocks; ++b) {
        uint64_t counter[ORACLE_MAX_RANK];
        uint64_t map[ORACLE_BLOCK];
        const uint64_t begin = b * ORACLE_BLOCK;
        const uint64_t end = begin + ORACLE_BLOCK < total ? begin + ORACLE_BLOCK : total;
        /* Odometer start: unravel `begin` over the old shape. */
        uint64_t rem = begin, pn = 0;
        for (int i = rank - 1; i >= 0; --i) {
            counter[i] = rem % shape[i];
            rem /= shape[i];
            pn += counter[i] * step[i];
        }
        for (uint64_t po = begin; po < end; ++po) {
            map[po - begin] = pn;
            /* Increment the odometer (Default.hpp:100-111). */
            for (int j = rank - 1; j >= 0; --j) {
                if (++counter[j] < shape[j]) {
                    pn += step[j];
                    break;
                }
                pn -= (shape[j] - 1) * step[j];
                counter[j] = 0;
            }
        }
        if (elem_bytes == 8) {
            const uint64_t *s = (const uint64_t *)src;
            uint64_t *d = (uint64_t *)dst;
            for (uint64_t po = begin; po < end; ++po)
                d[map[po - begin]] = s[po];
        }
        else {
            for (uint64_t po = begin; po < end; ++po)
                memcpy(dst + map[po - begin] * elem_bytes, src + po * elem_bytes,
                       (size_t)elem_bytes);
        }
    }
    (void)nthreads;
    return 0;
}

/* Number of OpenMP threads the port uses (1 without OpenMP). */
int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
