// irregular/ros.h -- the device reduction object an application's
// irregular.h inserts into (OBJECT = Sobject under GPU_KERNEL), with the
// reference's names and insert signature (moldyn/irregular/ros.h:5-27).
// The reference's object is a shared-memory hash table of NUM_BUCKETS_S
// keys merged into a global one per part; here it is one node's row (see
// irregular_plugin.cuh): inserts keyed by the row are combined with the
// application's reduce in entry order, other keys are dropped.  Defining
// IRR_PLUGIN_COMPENSATED before including it sums VALUE's floats with
// compensated (TwoSum) accumulators instead, for a reduce that is float +.
#ifndef REDUCTION_S
#define REDUCTION_S

#include "irregular_plugin.cuh"
#include "parameters.h"

namespace FGPU {
typedef void (*irreduce_fp)(VALUE *value1, VALUE *value2);
}

using namespace FGPU;

#ifdef IRR_PLUGIN_COMPENSATED
struct Reduction_Object_S : irr_plugin::RowSumObject<KEY, VALUE, FGPU::irreduce_fp> {};
#else
struct Reduction_Object_S : irr_plugin::RowObject<KEY, VALUE, FGPU::irreduce_fp> {};
#endif

typedef struct Reduction_Object_S Sobject;

#endif
