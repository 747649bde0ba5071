// irregular/parameters.h -- the types an application's irregular.h takes
// from the runtime (moldyn/irregular/parameters.h:17-28): KEY, the node id
// a map inserts under, and VALUE, its per-node reduction record.  An
// application with another VALUE puts its own irregular/parameters.h ahead
// of this directory on the include path (the reference's is edited in
// place); the guard name is the reference's, so only one is used.
#ifndef IRREGULAR_PARAMETERS_H_
#define IRREGULAR_PARAMETERS_H_

typedef int KEY;

struct value {
    float x;
    float y;
    float z;
};
typedef struct value VALUE;

#endif
