/* A user per-edge function in the reference's irregular.h form (the
 * DEVICE/OBJECT/CONSTANT switch, namespace FGPU, map and reduce tables of
 * moldyn/irregular.h:9-118), for the plugin tests: a harmonic spring of rest
 * length r0 and stiffness k between every listed pair closer than rcut,
 * f_i = -k (1 - r0 / r) d with d = x_i - x_j, in FP64, open boundaries;
 * +f to idx0, -f to idx1.  Table entry 1 is the same law scaled by 2 (to
 * check map_idx selection); reduce entry 0 adds, entry 1 keeps the
 * component-wise maximum (a reduce that is not +). */
#ifndef IRREGULAR_H_
#define IRREGULAR_H_
#include "irregular/parameters.h"
#include <math.h>
#include "irregular/ros.h"
#include "spring.h"

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

DEVICE bool spring_scaled(OBJECT *object, void *point_data, int *part_index, void *edge_data,
                          void *parameter, unsigned int task_id, unsigned int part_id,
                          irreduce_fp reduce_ptr, double scale)
{
    const struct spring_para *sp = (const struct spring_para *)parameter;
    const struct spring_node *nodes = (const struct spring_node *)point_data;
    const int *pair = (const int *)edge_data + 2 * task_id;
    int a = pair[0], b = pair[1];
    double d[3], r2 = 0.0;
    for (int c = 0; c < 3; c++) {
        d[c] = nodes[a].x[c] - nodes[b].x[c];
        r2 += d[c] * d[c];
    }
    if (!(r2 < sp->rcut * sp->rcut) || r2 == 0.0) return true;
    const double g = -scale * sp->k * (1.0 - sp->r0 / sqrt(r2));
    VALUE f;
    f.x = (float)(g * d[0]);
    f.y = (float)(g * d[1]);
    f.z = (float)(g * d[2]);
    if (part_index[a] == (int)part_id) object->insert(&a, &f, reduce_ptr);
    if (part_index[b] == (int)part_id) {
        f.x = -f.x;
        f.y = -f.y;
        f.z = -f.z;
        object->insert(&b, &f, reduce_ptr);
    }
    return true;
}

DEVICE bool spring(OBJECT *object, void *point_data, int *part_index, void *edge_data, void *parameter,
                   unsigned int task_id, unsigned int part_id, irreduce_fp reduce_ptr)
{
    return spring_scaled(object, point_data, part_index, edge_data, parameter, task_id, part_id,
                         reduce_ptr, 1.0);
}

DEVICE bool spring2(OBJECT *object, void *point_data, int *part_index, void *edge_data, void *parameter,
                    unsigned int task_id, unsigned int part_id, irreduce_fp reduce_ptr)
{
    return spring_scaled(object, point_data, part_index, edge_data, parameter, task_id, part_id,
                         reduce_ptr, 2.0);
}

DEVICE void add(VALUE *v1, VALUE *v2)
{
    v1->x += v2->x;
    v1->y += v2->y;
    v1->z += v2->z;
}

DEVICE void keep_max(VALUE *v1, VALUE *v2)
{
    v1->x = fmaxf(v1->x, v2->x);
    v1->y = fmaxf(v1->y, v2->y);
    v1->z = fmaxf(v1->z, v2->z);
}

CONSTANT irmap_fp map_function_table[] = {spring, spring2};
CONSTANT irreduce_fp reduce_function_table[] = {add, keep_max};
}

#endif
