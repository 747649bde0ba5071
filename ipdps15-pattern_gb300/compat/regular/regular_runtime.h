// regular/regular_runtime.h -- a host stand-in for the reference's
// generalized-reduction runtime (moldyn/regular/regular_runtime.h), which is a
// different pattern and outside this library.  The drivers construct it for
// their kinetic-energy / average-velocity summaries (moldyn/moldyn.cu:459-463,
// miniMD/ljs.cu:164-166) and print those from their own serial loops; this
// stand-in keeps the interface so they compile and link, and computes
// nothing (RegularGetOutput returns an empty output).
#ifndef REGULAR_RUNTIME_H_
#define REGULAR_RUNTIME_H_

#include <stddef.h>
#include <string.h>

struct element_t {
    size_t offset;
    size_t size;
};
typedef struct element_t Offset;

struct output {
    char *output_keys;
    char *output_vals;
    unsigned int *key_index;
    unsigned int *val_index;
    unsigned int key_num;
    unsigned int key_size;
    unsigned int value_size;
};

class RegularRuntime {
public:
    RegularRuntime(int num_procs, void *input, size_t input_size, Offset *offsets,
                   size_t offset_number, void *parameters, int parameter_size)
        : input_(input), input_size_(input_size), offsets_(offsets),
          num_offsets_(offset_number), parameter_(parameters), parameter_size_(parameter_size)
    {
        (void)num_procs;
        memset(&out_, 0, sizeof(out_));
    }
    void RegularInit() {}
    void RegularStart() {}
    struct output RegularGetOutput() { return out_; }
    void set_map_idx(int) {}
    void set_reduce_idx(int) {}

private:
    void *input_;
    size_t input_size_;
    Offset *offsets_;
    size_t num_offsets_;
    void *parameter_;
    int parameter_size_;
    struct output out_;
};

#endif
