/* plg_work.h — the algorithmic work of one Physics.update() per unit, in
 * which the roofline figures of this library are quoted (achieved rate =
 * these counts x the units a launch processes / the launch's duration).
 *
 * Bytes are the minimal DRAM traffic of each kernel by design (FP32
 * structure-of-arrays state: 2D position+type+id 16 B, velocity 8 B; 3D
 * position+type 16 B, velocity+id 16 B); flops count an FMA as 2, a
 * compare, a select-free clamp and an rsqrt as 1.  Header only, no code. */
#ifndef PLG_WORK_H
#define PLG_WORK_H

/* Whole step, per particle: read the sorted state, write the next state,
 * the cell key written and read once (cell-start tables are per cell and
 * negligible at the benchmark densities).  2D: 24 + 24 + 8; 3D: 32 + 32 + 8. */
#define PLG_WORK_STEP_BYTES_2D 56
#define PLG_WORK_STEP_BYTES_3D 72

/* k_force_tile, per particle: read B position+velocity, write A
 * position+velocity, write the new cell, read the target's cell from the
 * sort (2D: 24 + 24 + 4 + 4; 3D: 32 + 32 + 4 + 4). */
#define PLG_WORK_FORCE_BYTES_2D 56
#define PLG_WORK_FORCE_BYTES_3D 72

/* k_force_tile, per candidate pair (every pair of the 9 / 27-cell stencil):
 * the two (three) differences, d2 (one FMA per extra axis), and the decision
 * band compares: 2D 6, 3D 9. */
#define PLG_WORK_FLOPS_CANDIDATE_2D 6
#define PLG_WORK_FLOPS_CANDIDATE_3D 9

/* Per interacting pair, on top of its candidate work: rsqrt, distance,
 * the force law (two FMAs, abs-FMA, clamp, select, scale) and the
 * accumulation (one FMA per axis): 2D 13, 3D 15. */
#define PLG_WORK_FLOPS_INTERACTION_2D 13
#define PLG_WORK_FLOPS_INTERACTION_3D 15

/* Sort kernels.  k_scan per cell: read the count, write the start.
 * k_scatter per particle: read the cell and its start, the rank taken from
 * the counts, write the permutation entry and the slot's cell.
 * k_gather per particle: permutation and slot cell, the cell's two starts,
 * the old state (24 B in 2D), the new state, and the in-cell re-rank reads. */
#define PLG_WORK_SCAN_BYTES_PER_CELL 8
#define PLG_WORK_SCATTER_BYTES 16
#define PLG_WORK_GATHER_BYTES_2D 64

#endif
