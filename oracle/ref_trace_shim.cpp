// C entry points over the reference's own CPU integrator -- TEST INFRASTRUCTURE ONLY.
// Compiled by oracle/Makefile from the reference's unmodified src/physics/Geodesic.h (found
// through -I<reference>/src) into oracle/_ref/libbhs_ref.so. Used to generate golden vectors
// (tests/golden/make_golden.py) and to pin the restatement in oracle/march.hpp against the
// reference itself.
#include <cstring>

#include "physics/Geodesic.h"

extern "C" {

// bhs::physics::trace (Geodesic.h:107-140). out9: dir[3] (TraceResult::dir), and the
// impact parameter / axis values of the same ray: impactParameter, impactParameterAboutAxis(+Y),
// shadowAngularRadius(|cam|), then 3 zeros. out_int: status (Escaped 0, Captured 1,
// MaxSteps 2), steps, equatorCrossings. out_minr: minR.
int ref_trace(const double cam[3], const double dir[3], int max_steps, double step_scale, double esc_tol,
              double r_esc_min, double* out9, int* out_int, double* out_minr) {
    const glm::dvec3 c(cam[0], cam[1], cam[2]);
    const glm::dvec3 d(dir[0], dir[1], dir[2]);
    const bhs::physics::TraceResult r = bhs::physics::trace(c, d, max_steps, step_scale, esc_tol, r_esc_min);
    out9[0] = r.dir.x;
    out9[1] = r.dir.y;
    out9[2] = r.dir.z;
    out9[3] = bhs::physics::impactParameter(c, d);
    out9[4] = bhs::physics::impactParameterAboutAxis(c, d, glm::dvec3(0.0, 1.0, 0.0));
    out9[5] = bhs::physics::shadowAngularRadius(glm::length(c));
    out9[6] = out9[7] = out9[8] = 0.0;
    out_int[0] = static_cast<int>(r.status);
    out_int[1] = r.steps;
    out_int[2] = r.equatorCrossings;
    *out_minr = r.minR;
    return 0;
}

// One rk4Step (Geodesic.h:27-34) and one initialVelocity / farFieldDirection evaluation.
void ref_rk4_step(double x[3], double v[3], double h2, double dt) {
    glm::dvec3 X(x[0], x[1], x[2]), V(v[0], v[1], v[2]);
    bhs::physics::rk4Step(X, V, h2, dt);
    x[0] = X.x; x[1] = X.y; x[2] = X.z;
    v[0] = V.x; v[1] = V.y; v[2] = V.z;
}
void ref_initial_velocity(const double cam[3], const double dir[3], double out[3]) {
    const glm::dvec3 r = bhs::physics::initialVelocity(glm::dvec3(cam[0], cam[1], cam[2]), glm::dvec3(dir[0], dir[1], dir[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void ref_far_field(const double x[3], const double v[3], double h2, double out[3]) {
    const glm::dvec3 r = bhs::physics::farFieldDirection(glm::dvec3(x[0], x[1], x[2]), glm::dvec3(v[0], v[1], v[2]), h2);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

// redshiftFactor (Geodesic.h:90-95), the CPU mirror of the disk shader's factor
double ref_redshift_factor(double r_emit, double b_axis, double r_cam) {
    return bhs::physics::redshiftFactor(r_emit, b_axis, r_cam);
}

}  // extern "C"
