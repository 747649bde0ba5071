/* Node record and parameter block of the spring plugin (tests/plugin/spring/
 * irregular.h): 32-byte nodes (position and a mass the map ignores, to check
 * records that are not bare positions), FP64 parameters. */
#ifndef SPRING_H_
#define SPRING_H_
struct spring_node {
    double x[3];
    double mass;
};
struct spring_para {
    double k;
    double r0;
    double rcut;
};
#endif
