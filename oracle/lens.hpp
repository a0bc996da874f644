// CPU restatement of the reference's lens-table builder -- TEST INFRASTRUCTURE ONLY.
//
//   shaders/gas_lens.glsl:13-21   LENS_RAYS, LENS_PHIS, LENS_RMAX, LENS_P, lensAlpha
//   shaders/gas_lens.comp:10-43   one ray of the fan: RK4 with ds = (r < 8 ? 0.004 : 0.01) r,
//                                 log r linearly interpolated at swept angles j 2 pi / 1023,
//                                 clamped to log 2, filled after capture / escape
// Table layout as the reference's image (x = ray, y = angle): table[j * 1024 + i].
#pragma once
#include <cmath>

#include "march.hpp"

namespace oracle {

constexpr int kLensRays = 1024, kLensPhis = 1024;

template <class T> inline T lensAlpha(T u, T ac) {
    const T pi = T(3.14159265358979);
    const T uc = ac / pi;
    if (u < uc) return ac - ac * std::pow((uc - u) / uc, T(3));
    return ac + (pi - ac) * std::pow((u - uc) / (T(1) - uc), T(3));
}

template <class T> inline void lensRay(int i, T camR, T ac, float* table) {
    const T two_pi = T(6.28318530717959), r_h = T(2), rmax = T(2.0e5);
    const T a = lensAlpha((T(i) + T(0.5)) / T(kLensRays), ac);
    V3<T> x{camR, T(0), T(0)};
    V3<T> v = initialVelocity(x, V3<T>{-std::cos(a), std::sin(a), T(0)});
    const V3<T> hv = cross(x, v);
    const T h2 = dot(hv, hv);
    const T dphi_j = two_pi / T(kLensPhis - 1);
    const T logH = std::log(r_h);
    table[i] = float(std::log(camR));
    int j = 1;
    T phi = T(0), r = camR;
    for (int s = 0; s < 20000 && j < kLensPhis; ++s) {
        const T ds = (r < T(8) ? T(0.004) : T(0.01)) * r;
        const V3<T> x0 = x;
        const T r0 = r;
        rk4Step(x, v, h2, ds / length(v));
        r = length(x);
        const T dphi = std::atan2(x0.x * x.y - x0.y * x.x, x0.x * x.x + x0.y * x.y);
        const T phi1 = phi + dphi;
        for (; j < kLensPhis && T(j) * dphi_j <= phi1; ++j) {
            const T t = std::min(std::max((T(j) * dphi_j - phi) / std::max(dphi, T(1e-12)), T(0)), T(1));
            table[size_t(j) * kLensRays + i] = float(std::max(std::log(r0 * (T(1) - t) + r * t), logH));
        }
        phi = phi1;
        if (r < r_h + T(0.01) || (r > rmax && dot(x, v) > T(0))) break;
    }
    const T fill = r < T(10) ? logH : std::log(rmax);
    for (; j < kLensPhis; ++j) table[size_t(j) * kLensRays + i] = float(fill);
}

}  // namespace oracle
