// irregular/irr_user_map.cu -- the translation unit an application adds to
// its build to run its own irregular.h on the GB300 library (the reference
// compiles the same file into its gpu_kernel.cu, moldyn/irregular/
// gpu_kernel.cu:1-10).  Compile it with nvcc for sm_103a, the application's
// directory (irregular.h and the headers it includes) and this compat
// directory on the include path, the application's directory holding no
// irregular/ subdirectory of its own:
//   nvcc -gencode arch=compute_103a,code=sm_103a -I <app> -I <compat>
//        -I <include> -c irr_user_map.cu
// It exports
//   irr_compat_user_launch        the launch function (irr_user_launch_fn):
//                                 map_function_table[map_idx] and
//                                 reduce_function_table[reduce_idx] of the
//                                 application's FGPU namespace, one thread per
//                                 node row;
//   irr_compat_register_user_map  binds it to a handle (the compat
//                                 IrregularRuntime calls it), VALUE records of
//                                 sizeof(VALUE) bytes, IRR_VALUE_F32 unless
//                                 IRR_PLUGIN_VALUE_KIND says otherwise.
#ifndef GPU_KERNEL
#define GPU_KERNEL
#endif
#include "irregular.h"

#include "irregular_gb300.h"
#include "irregular_plugin.cuh"

#ifndef IRR_PLUGIN_VALUE_KIND
#define IRR_PLUGIN_VALUE_KIND IRR_VALUE_F32
#endif

namespace {

struct TableCall {
    int map_idx;
    int reduce_idx;
    __device__ void operator()(Sobject *object, void *point_data, int *part_index, void *edge_data,
                               void *parameter, unsigned int task_id, unsigned int part_id) const
    {
        FGPU::map_function_table[map_idx](object, point_data, part_index, edge_data, parameter, task_id,
                                          part_id, FGPU::reduce_function_table[reduce_idx]);
    }
};

// IRR_PLUGIN_INLINE_MAP=<name>: call that map of the FGPU namespace directly
// (inlined into the kernel) instead of through the table; map_idx is then
// ignored.  With IRR_PLUGIN_COMPENSATED the reduce is not called either.
#ifdef IRR_PLUGIN_INLINE_MAP
struct InlineCall {
    int reduce_idx;
    __device__ void operator()(Sobject *object, void *point_data, int *part_index, void *edge_data,
                               void *parameter, unsigned int task_id, unsigned int part_id) const
    {
        FGPU::IRR_PLUGIN_INLINE_MAP(object, point_data, part_index, edge_data, parameter, task_id, part_id,
                                    FGPU::reduce_function_table[reduce_idx]);
    }
};
#endif

constexpr int kNumMaps = (int)(sizeof(FGPU::map_function_table) / sizeof(FGPU::map_function_table[0]));
constexpr int kNumReduces =
    (int)(sizeof(FGPU::reduce_function_table) / sizeof(FGPU::reduce_function_table[0]));

}  // namespace

extern "C" int irr_compat_user_launch(const irr_user_view *view, void *stream, void *ctx)
{
    (void)ctx;
    if (!view || view->map_idx < 0 || view->map_idx >= kNumMaps || view->reduce_idx < 0 ||
        view->reduce_idx >= kNumReduces)
        return IRR_ERR_ARG;
#ifdef IRR_PLUGIN_INLINE_MAP
    return irr_plugin::launch_rows<Sobject>(view, stream, InlineCall{view->reduce_idx});
#else
    return irr_plugin::launch_rows<Sobject>(view, stream, TableCall{view->map_idx, view->reduce_idx});
#endif
}

extern "C" int irr_compat_register_user_map(irr_handle *h)
{
    return irr_set_user_map(h, irr_compat_user_launch, nullptr, (int)sizeof(VALUE), IRR_PLUGIN_VALUE_KIND);
}
