/* Parameter block of the box entry of tests/plugin/lj/irregular.h: the
 * layout of moldyn's struct para (moldyn/moldyn.h:39-43). */
#ifndef LJDEFS_H_
#define LJDEFS_H_
struct lj_box_para {
    double side;
    double cutoff;
};
#endif
