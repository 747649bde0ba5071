/* The Lennard-Jones law of the reference's two drivers, written as a user
 * per-edge function in the irregular.h form (moldyn/irregular.h:9-118), for
 * the plugin tests.  Both entries evaluate, in FP64, the pair force divided
 * by 48 at eps = sigma = 1, d (r^-14 - r^-8 / 2) with d = x_i - x_j, for
 * r^2 below the squared cutoff, and insert +f (rounded to float) under idx0
 * and -f under idx1:
 *   entry 0: minimum image in a cubic box, parameters {side, cutoff radius}
 *            (moldyn `map`, moldyn/irregular.h:26-107);
 *   entry 1: open boundaries, parameter cutoff^2 (miniMD `map1`,
 *            miniMD/irregular.h:109-163).
 * Nodes are FP64 xyz triples (moldyn's point_data, miniMD's nodes). */
#ifndef IRREGULAR_H_
#define IRREGULAR_H_
#include "irregular/parameters.h"
#include <math.h>
#include "irregular/ros.h"
#include "ljdefs.h"

#if defined(GPU_KERNEL)
#define DEVICE __device__
#define OBJECT Sobject
#define CONSTANT __constant__
namespace FGPU
{
#elif defined(CPU_KERNEL)
#define DEVICE
#define OBJECT Cobject
#define CONSTANT
namespace FCPU
{
#endif
typedef void (*irreduce_fp)(VALUE *value1, VALUE *value2);
typedef bool (*irmap_fp)(OBJECT *object, void *point_data, int *part_index, void *edge_data,
                         void *parameter, unsigned int task_id, unsigned int part_id,
                         irreduce_fp reduce_ptr);

DEVICE void lj_insert(OBJECT *object, int *part_index, unsigned int part_id, int a, int b,
                      const double d[3], double rr, irreduce_fp reduce_ptr)
{
    const double inv = 1.0 / rr;
    const double inv2 = inv * inv;
    const double inv4 = inv2 * inv2;
    const double s = inv4 * inv2 * inv - 0.5 * inv4; /* r^-14 - r^-8 / 2 */
    VALUE f;
    f.x = (float)(d[0] * s);
    f.y = (float)(d[1] * s);
    f.z = (float)(d[2] * s);
    if (part_index[a] == (int)part_id) object->insert(&a, &f, reduce_ptr);
    if (part_index[b] == (int)part_id) {
        f.x = -f.x;
        f.y = -f.y;
        f.z = -f.z;
        object->insert(&b, &f, reduce_ptr);
    }
}

DEVICE bool lj_box(OBJECT *object, void *point_data, int *part_index, void *edge_data, void *parameter,
                   unsigned int task_id, unsigned int part_id, irreduce_fp reduce_ptr)
{
    const struct lj_box_para *bp = (const struct lj_box_para *)parameter;
    const double *x = (const double *)point_data;
    const int *pair = (const int *)edge_data + 2 * task_id;
    const int a = pair[0], b = pair[1];
    const double half = 0.5 * bp->side;
    double d[3];
    for (int c = 0; c < 3; c++) {
        double v = x[3 * a + c] - x[3 * b + c];
        if (v < -half) v += bp->side;
        if (v > half) v -= bp->side;
        d[c] = v;
    }
    const double rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (rr < bp->cutoff * bp->cutoff) lj_insert(object, part_index, part_id, a, b, d, rr, reduce_ptr);
    return true;
}

DEVICE bool lj_open(OBJECT *object, void *point_data, int *part_index, void *edge_data, void *parameter,
                    unsigned int task_id, unsigned int part_id, irreduce_fp reduce_ptr)
{
    const double cut2 = *(const double *)parameter;
    const double *x = (const double *)point_data;
    const int *pair = (const int *)edge_data + 2 * task_id;
    const int a = pair[0], b = pair[1];
    double d[3];
    for (int c = 0; c < 3; c++) d[c] = x[3 * a + c] - x[3 * b + c];
    const double rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (rr < cut2) lj_insert(object, part_index, part_id, a, b, d, rr, reduce_ptr);
    return true;
}

DEVICE void add3(VALUE *v1, VALUE *v2)
{
    v1->x += v2->x;
    v1->y += v2->y;
    v1->z += v2->z;
}

CONSTANT irmap_fp map_function_table[] = {lj_box, lj_open};
CONSTANT irreduce_fp reduce_function_table[] = {add3};
}

#endif
