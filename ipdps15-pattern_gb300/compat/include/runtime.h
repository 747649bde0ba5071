// include/runtime.h -- the reference's runtime entry points
// (moldyn/include/runtime.h, runtime.cpp:4-12).  One process drives one GPU:
// there is no MPI world to initialise, so both are no-ops.
#ifndef INCLUDE_RUNTIME_H_
#define INCLUDE_RUNTIME_H_

static inline void RuntimeInit(int argc, char *argv[])
{
    (void)argc;
    (void)argv;
}
static inline void RuntimeFinalize() {}

#endif
