/*
 * irr_oracle.h -- CPU oracle for the irregular-reduction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs use it, and only as the reference
 * results they compare against or as the timed CPU baseline.
 *
 * It restates, in plain C, the arithmetic of the reference's CPU path:
 *   - the per-edge user function `map` (moldyn/irregular.h:26-107) and
 *     `map1` (miniMD/irregular.h:109-163), with the `reduce` float3 `+=`
 *     (moldyn/irregular.h:109-114);
 *   - the pthread executor `compute_cpu` (moldyn/irregular/cpu_kernel.cu:13-70)
 *     with its per-thread open-addressing table `Cobject::insert`
 *     (moldyn/irregular/roc.cu:11-65), used as the timed CPU baseline;
 *   - the binned half neighbour list of miniMD (miniMD/neighbor.cpp:76-205)
 *     and the all-pairs list rule of moldyn (moldyn/moldyn.cu:552-594);
 *   - the GPU partitioner's Morton ordering and edge binning, which has no
 *     reference counterpart beyond the part bookkeeping of
 *     moldyn/irregular/partitioner.cpp:142-297; the oracle fixes the exact
 *     integer results the GPU pass must reproduce bit for bit.
 *
 * Parity pinning: the restated `map`/`map1` numerics are checked against the
 * reference's own FCPU::map compiled from its sources (oracle/ref_harness.cpp,
 * built into oracle/_ref/), and the neighbour builders against the two known
 * list sizes the reference logs (miniMD/2:13 and moldyn/irresult/2:5).
 */
#ifndef IRR_ORACLE_H_
#define IRR_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Lennard-Jones law in the reference's form r*(r^-14 - r^-8/2) (the LJ force
 * divided by 48 at eps = sigma = 1).  periodic != 0 selects moldyn's minimum
 * image (moldyn/irregular.h:51-60) with box side `side`; cutoff2 is the
 * squared force cutoff compared with `<` (moldyn/irregular.h:64,
 * miniMD/irregular.h:133). */
typedef struct {
    double side;
    double cutoff2;
    int periodic;
} orc_lj_param;

/* FP64 reduction over all edges (the oracle).  pos: 3n doubles.  f: 3n out.
 * sabs (optional): per node and component, the sum over incident in-cutoff
 * edges of |d_c| * (r^-14 + r^-8/2) -- the magnitude of the terms before
 * cancellation, used as the per-node error scale. */
void orc_lj_edge_scale_inf(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                           const orc_lj_param *p, double *sinf);
void orc_lj_reduce_f64(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                       const orc_lj_param *p, double *f, double *sabs);

/* The reference's CPU numerics, single-threaded and deterministic: per edge
 * the FP64 `map` result is rounded to float (VALUE is float3,
 * moldyn/irregular/parameters.h:21-28) and added with float `+=` in edge
 * order, +f to idx0 and -f to idx1. */
void orc_lj_reduce_refnum_f32(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                              const orc_lj_param *p, float *f);

/* Port of the reference's CPU executor (moldyn/irregular/cpu_kernel.cu:13-70):
 * `threads` workers take `chunk` consecutive edges at a time from a
 * mutex-guarded cursor, run the FP64 per-edge law and insert both endpoint
 * contributions into a private open-addressing table with a per-bucket CAS
 * lock and linear probing (moldyn/irregular/roc.cu:11-65).  Table set-up is
 * excluded from the timing, as re_init is in the reference.  The tables are
 * then merged in thread order into f (the reference's merge is a no-op,
 * roc.cu:67-77, so the harness merges).  Returns 0 on success; *seconds gets
 * the fork-to-join wall time (irregular_runtime.cu:286-301). */
int orc_cpu_executor(int64_t n, const double *pos, int64_t e, const int32_t *edges,
                     const orc_lj_param *p, int threads, int64_t chunk, float *f,
                     double *seconds);

/* Same executor over float xyz positions (12 B per node) and a caller-owned
 * set of tables, so a benchmark can time repeated passes without
 * re-allocating.  Returns seconds of the fork-to-join region, < 0 on error. */
typedef struct orc_exec orc_exec;
orc_exec *orc_exec_create(int64_t n, int threads);
double orc_exec_run(orc_exec *x, const float *pos, int64_t e, const int32_t *edges,
                    const orc_lj_param *p, int64_t chunk, float *f_out);
void orc_exec_destroy(orc_exec *x);

/* Half neighbour list by cell binning.  pos: 3n floats.  box > 0 selects
 * periodic minimum image with side `box`; box == 0 is open boundaries
 * (miniMD builds no ghosts, miniMD/neighbor.cpp:76-205).  A pair i<j is
 * listed when r2 <= list_cut2, r2 evaluated in float as
 * ((dx*dx + dy*dy) + dz*dz) with each operation rounded (no FMA), d wrapped
 * once by +-box when |d| > box/2.  Output pairs are (i, j), i < j, sorted by
 * i then j.  Returns the pair count; writes at most cap pairs when out is
 * non-NULL.  Returns -1 on bad arguments. */
int64_t orc_neighbor_half_list(int64_t n, const float *pos, float box, float list_cut2,
                               int32_t *out, int64_t cap);

/* The same list restricted to rows i in [row_begin, row_end) (pairs i < j,
 * j anywhere): a bounded sample of a large list for the timed CPU baseline. */
int64_t orc_neighbor_half_list_rows(int64_t n, const float *pos, float box, float list_cut2,
                                    int64_t row_begin, int64_t row_end, int32_t *out, int64_t cap);

/* FP64 reference MD for the GPU loop: velocity Verlet (m = 1), forces
 * 48 d (r^-14 - r^-8/2) for pairs inside `cutforce` with moldyn's minimum
 * image, positions wrapped into [0, side) after each drift, the half list
 * (orc_neighbor_half_list on the float copy of the positions, cutoff
 * cutforce + skin) rebuilt after the drift of every rebuild_every-th step.
 * pos, vel: 3n doubles, updated in place.  ke / pe (optional) receive the
 * final kinetic and potential (4(r^-12 - r^-6) inside the cutoff) energy. */
int orc_md_run_mt(int64_t n, double *pos, double *vel, double side, double cutforce, double skin,
                  double dt, int steps, int rebuild_every, double *ke, double *pe, int threads,
                  int float_forces);
int orc_md_run(int64_t n, double *pos, double *vel, double side, double cutforce, double skin,
               double dt, int steps, int rebuild_every, double *ke, double *pe);

/* FCC lattice of moldyn's InitCoordinates (moldyn/moldyn.cu:596-626):
 * 4*m^3 points, spacing side/m.  pos: 3*4*m^3 doubles. */
void orc_fcc_moldyn(int m, double side, double *pos);
/* FCC lattice of miniMD's create_atoms (miniMD/setup.cpp:61-122) for an
 * nx*ny*nz cell box at density rho; returns the atom count written. */
int64_t orc_fcc_minimd(int nx, int ny, int nz, double rho, double *pos, int64_t cap);

/* Partition oracle.  Morton key of each node from float positions: per axis
 * q = trunc((x - lo) * scale) clamped to [0, 1023] (float ops, each rounded),
 * key = bit interleave of (qx, qy, qz), x in the lowest bit. */
void orc_morton_keys(int64_t n, const float *pos, const float lo[3], const float scale[3],
                     uint32_t *keys);
/* Full partition: stable sort by key (ties by node id) gives perm[new]=old
 * and inv[old]=new; every half edge (i, j) at list position t yields the
 * directed entries (inv[i] <- inv[j]) and (inv[j] <- inv[i]); binning all
 * entries by row gives row_off[n+1], and each row's columns are sorted
 * ascending, so col[2e] is in (row, col) order whatever the edge order. */
int orc_partition(int64_t n, const float *pos, const float lo[3], const float scale[3],
                  int64_t e, const int32_t *edges, int32_t *perm, int32_t *inv,
                  int64_t *row_off, int32_t *col);
/* Hilbert keys on the same 10-bit grid (Skilling's transposed index, axis 0
 * in the high bit of each 3-bit group), and the partition ordered by either
 * curve: curve 0 = Hilbert, 1 = Morton (orc_partition). */
void orc_hilbert_keys(int64_t n, const float *pos, const float lo[3], const float scale[3],
                      uint32_t *keys);
int orc_partition_curve(int64_t n, const float *pos, const float lo[3], const float scale[3],
                        int curve, int64_t e, const int32_t *edges, int32_t *perm, int32_t *inv,
                        int64_t *row_off, int32_t *col);

/* Staged ("halo") entry layout of a CSR (rows in execution order, columns
 * ascending), for 4 lanes per row and slices of 8 rows -- the GPU builder's
 * output, bit for bit.  No reference counterpart: it restates the library's
 * own layout so that the GPU pass is checked as integer work.
 *   Cut: the rows are taken 8 at a time in order (block q: rows [8q, 8q + 8),
 *     clipped to n, taking 32 (T + 1) words with T = its longest row's entries
 *     / 8 rounded up); the blocks are cut greedily into runs of at most
 *     slices_per_item blocks and stream_max words; each run is then cut
 *     greedily into the longest prefixes whose table -- the sorted distinct
 *     ids of the item's rows and of all their columns -- holds at most tab_max
 *     ids.  An item of rows [r0, r0 + m) covers ceil(m / 8) slices.
 *   Slices: within an item the rows are ordered by entry count, longest
 *     first (ties by row id), and slice j of the item takes rows 8j .. 8j + 7
 *     of that order (positions past m are padding rows), so that rows of a
 *     slice have similar lengths; slice j takes 32 (T_j + 1) words, T_j = its
 *     longest row's entries / 8 rounded up (never more words than the cut
 *     counted).  slice_off holds each slice's first word.
 *   Words of a slice: word 4i + l (row i, lane l) of its first 32 is the
 *     header own | len << 14 | lrow << 24 (own: the byte offset 16 * slot of
 *     the row's own id in the item's table; len < 1024; lrow = row - r0); a
 *     padding row's header is 1 << 31; word 32 (t + 1) + 4i + l is
 *     b0 | b1 << 16, the byte offsets of the row's picks (t, 0, l) and
 *     (t, 1, l).  Row i (parity p = i & 1) picks in the order
 *     (t, h, l): from bank group g = (2t + h + 4p + l) mod 8 (a slot's group is
 *     slot mod 8) its lowest remaining entry; if that group is empty, from the
 *     group with the most remaining entries (the lowest such group); when
 *     none remain, its own slot (padding, masked by len in the kernel).
 * Outputs may be NULL (sizes only).  items: 6 int32 per item (row0, nrows,
 * word0, nwords, tab0, ntab).  Returns 0, or -1 when a slice alone exceeds
 * stream_max words or tab_max ids (the layout does not apply), -2 on bad
 * arguments. */
int orc_staged_layout(int64_t n, const int64_t *row_off, const int32_t *col, int slices_per_item,
                      int tab_max, int stream_max, int64_t *num_items, int64_t *num_words,
                      int64_t *num_ids, int32_t *items, uint32_t *slice_off, uint32_t *words,
                      int32_t *ids);

#ifdef __cplusplus
}
#endif
#endif
