// wf_setup.h — host domain set-up helpers (generators, zones), C ABI.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
int64_t wf_gen_cylinder(double x0, double y0, double z0, double Rxy, double Lz, double r,
                        double density, double* x, double* mass);
int64_t wf_gen_box(double x0, double y0, double z0, double Lx, double Ly, double Lz, double r,
                   double density, double* x, double* mass);
int64_t wf_gen_cylinder_lattice(double R, double H, double dx, double jitter, uint64_t seed,
                                double* x);
int64_t wf_assign_zone(const double* x, int64_t n, const double* start, const double* end,
                       int32_t zone_id, int32_t* id, uint8_t* not_write);
#ifdef __cplusplus
}
#endif
