// irregular/irregular_runtime.h -- drop-in replacement for the reference's
// IrregularRuntime (moldyn/irregular/irregular_runtime.h:12-112), implemented
// on the GB300 library's C ABI (irregular_gb300.h).  A driver that includes
// "irregular/irregular_runtime.h" compiles unchanged when this directory is
// ahead of the reference's own on the include path; link with
// -lirregular_gb300.
//
// Behaviour differences from the reference (all deliberate):
//  * one process, one GPU: MPI ranks, the CPU/GPU split and per-iteration
//    re-splits do not exist; IrregularBarrier is a stream synchronisation;
//  * the caller's edge and coordinate arrays are never modified, and results
//    come back in the caller's node order;
//  * the per-edge user function is the application's own irregular.h,
//    compiled by irregular/irr_user_map.cu (which the application adds to its
//    build, as the reference compiles irregular.h into its executors) and
//    bound by irr_compat_register_user_map; set_map_idx / set_reduce_idx pick
//    entries of its tables.  Defining IRR_COMPAT_MAP (an enum irr_map value)
//    instead selects one of the library's built-in laws, whose tiled kernel
//    is the fast path.  Without either the program does not link;
//  * the result buffer is read at reduction_elm_size bytes per node: VALUE
//    records, or their floats widened to doubles when reduction_elm_size is
//    twice sizeof(VALUE) (moldyn passes 3 doubles, moldyn/moldyn.cu:321);
//  * failures print the library's message and abort (the reference exit()s).
#ifndef IRREGULAR_IRREGULAR_RUNTIME_H_
#define IRREGULAR_IRREGULAR_RUNTIME_H_

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "irregular_gb300.h"

#ifndef IRR_COMPAT_MAP
// irregular/irr_user_map.cu: binds the application's irregular.h tables.
extern "C" int irr_compat_register_user_map(irr_handle *h);
#endif

typedef int64_t IRIndex;

#ifndef IRREGULAR_DATA_TYPE_H_
#define IRREGULAR_DATA_TYPE_H_
struct edge {
    int idx0;
    int idx1;
};
struct part {
    int start;
    int end;
    int part_id;
};
typedef struct part Part;
typedef struct edge EDGE;
#endif

class IrregularRuntime {
public:
    IrregularRuntime(IRIndex num_edges, IRIndex num_nodes, EDGE *edges, void *edge_data,
                     void *node_data, int edge_data_elm_size, int node_data_elm_size,
                     int reduction_elm_size, int node_num_dims, void *node_coordinates,
                     int coordinate_size, void *parameter, int parameter_size, int num_procs,
                     int num_iters)
        : num_edges_(num_edges), num_nodes_(num_nodes), node_elm_(node_data_elm_size),
          red_elm_(reduction_elm_size)
    {
        (void)edge_data;
        (void)edge_data_elm_size;
        (void)num_procs;
        (void)num_iters;
        irr_config cfg;
        irr_config_default(&cfg);
#ifdef IRR_COMPAT_MAP
        (void)node_num_dims;
        (void)node_coordinates;
        (void)coordinate_size;
        cfg.map_idx = IRR_COMPAT_MAP;
        check(irr_create(&cfg, &h_), "create");
#else
        check(irr_create(&cfg, &h_), "create");
        check(irr_compat_register_user_map(h_), "user map");
        if (node_coordinates)
            check(irr_set_coordinates(h_, node_coordinates, coordinate_size, node_num_dims, num_nodes),
                  "coordinates");
#endif
        check(irr_set_params(h_, parameter, parameter_size), "parameters");
        check(irr_set_edges(h_, (const int32_t *)edges, num_edges), "edges");
        check(irr_set_nodes(h_, node_data, node_data_elm_size, num_nodes), "node data");
    }

    ~IrregularRuntime()
    {
        if (h_) irr_destroy(h_);
    }

    void IrregularInit() { check(irr_init(h_), "IrregularInit"); }
    void IrregularStart() { check(irr_step(h_), "IrregularStart"); }
    void IrregularBarrier() { check(irr_sync(h_), "IrregularBarrier"); }
    void reset_node_data(void *node_data)
    {
        check(irr_set_nodes(h_, node_data, node_elm_, num_nodes_), "reset_node_data");
    }
    void get_reduction_result(void *buffer)
    {
        check(irr_get_result(h_, buffer, red_elm_), "get_reduction_result");
    }
    void set_map_idx(int idx) { check(irr_set_map(h_, idx), "set_map_idx"); }
    void set_reduce_idx(int idx) { check(irr_set_reduce(h_, idx), "set_reduce_idx"); }

    // the handle, for callers that also want the C ABI (streams, info, ...)
    irr_handle *handle() { return h_; }

private:
    IrregularRuntime(const IrregularRuntime &);
    IrregularRuntime &operator=(const IrregularRuntime &);

    void check(int rc, const char *what)
    {
        if (rc != IRR_OK) {
            fprintf(stderr, "IrregularRuntime %s: %s (%s)\n", what, irr_status_string(rc),
                    h_ ? irr_last_error(h_) : "");
            abort();
        }
    }

    irr_handle *h_ = nullptr;
    IRIndex num_edges_;
    IRIndex num_nodes_;
    int node_elm_;
    int red_elm_;
};

#endif
