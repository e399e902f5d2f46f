// Orbital elements of the binary for the minidisk time series: the host-side
// FP64 two_body::recover_orbital_elements (src/physics_two_body.hpp:284-379,
// G = 1) and the element rates implied by the gas's forces and accretion.
// Host code only; it runs once per time-series sample.
#include <algorithm>
#include <cmath>
#include <cstring>
#include "common.cuh"

namespace {

// recover_orbital_elements in the reference's order of operations.
// s = {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2}; false if not bound.
bool elements(const double* s, double t, double* out)
{
    const double G = 1.0;
    const double M1 = s[0], M2 = s[5];
    const double M = M1 + M2;
    const double q = M2 / M1;

    const double x_cm = (s[1] * M1 + s[6] * M2) / M;
    const double y_cm = (s[2] * M1 + s[7] * M2) / M;
    const double vx_cm = (s[3] * M1 + s[8] * M2) / M;
    const double vy_cm = (s[4] * M1 + s[9] * M2) / M;

    const double x1 = s[1] - x_cm, y1 = s[2] - y_cm;
    const double x2 = s[6] - x_cm, y2 = s[7] - y_cm;
    const double r1 = std::sqrt(x1 * x1 + y1 * y1);
    const double r2 = std::sqrt(x2 * x2 + y2 * y2);
    const double vx1 = s[3] - vx_cm, vy1 = s[4] - vy_cm;
    const double vx2 = s[8] - vx_cm, vy2 = s[9] - vy_cm;
    const double vf1 = -vx1 * y1 / r1 + vy1 * x1 / r1;
    const double vf2 = -vx2 * y2 / r2 + vy2 * x2 / r2;
    const double v1 = std::sqrt(vx1 * vx1 + vy1 * vy1);

    const double E1 = 0.5 * M1 * (vx1 * vx1 + vy1 * vy1);
    const double E2 = 0.5 * M2 * (vx2 * vx2 + vy2 * vy2);
    const double L1 = M1 * r1 * vf1;
    const double L2 = M2 * r2 * vf2;
    const double R = r1 + r2;
    const double L = L1 + L2;
    const double E = E1 + E2 - G * M1 * M2 / R;
    if (!(E < 0.0)) return false;

    const double a = -0.5 * G * M1 * M2 / E;
    const double b = std::sqrt(-0.5 * L * L / E * (M1 + M2) / (M1 * M2));
    const double e = std::sqrt(std::clamp(1.0 - b * b / a / a, 0.0, 1.0));
    const double omega = std::sqrt(G * M / a / a / a);

    const double a1 = a * q / (1.0 + q);
    const double b1 = b * q / (1.0 + q);

    const double cn = e == 0.0 ? x1 / r1 : (1.0 - r1 / a1) / e;
    const double cf = a1 / r1 * (cn - e);
    const double sn = e == 0.0 ? y1 / r1 : (vx1 * x1 + vy1 * y1) / (e * v1 * r1) * std::sqrt(1.0 - e * e * cn * cn);
    const double sf = (b1 / r1) * sn;

    const double cE = (e + cf) / (1.0 + e * cf);
    const double sE = std::sqrt(1.0 - e * e) * sf / (1.0 + e * cf);

    const double EA = std::atan2(sE, cE);
    const double MA = EA - e * sE;
    const double tau = t - MA / omega;

    const double ax = +(cn - e) * x1 + sn * std::sqrt(1.0 - e * e) * y1;
    const double ay = +(cn - e) * y1 - sn * std::sqrt(1.0 - e * e) * x1;
    const double pomega = std::atan2(ay, ax);

    const double v[10] = {a, M, q, e, x_cm, y_cm, vx_cm, vy_cm, pomega, tau};
    std::memcpy(out, v, sizeof v);
    return true;
}

} // namespace

extern "C" {

int mara_two_body_elements(const double* state, double time, double* out)
{
    MARA_REQUIRE(state && out, "mara_two_body_elements: null buffer");
    MARA_REQUIRE(state[0] > 0.0 && state[5] > 0.0, "mara_two_body_elements: masses must be positive");
    MARA_REQUIRE(elements(state, time, out), "two_body::recover_orbital_elements (not a bound orbit)");
    return MARA_OK;
}

int mara_two_body_element_rates(const double* state, double time, const double* rates, double* out)
{
    MARA_REQUIRE(state && rates && out, "mara_two_body_element_rates: null buffer");
    MARA_REQUIRE(state[0] > 0.0 && state[5] > 0.0, "mara_two_body_element_rates: masses must be positive");
    // d/dt of the state: masses grow by the sink mass rates; momenta by the
    // gas's gravity plus the sink momentum rates; positions are held.
    double ds[10] = {};
    for (int k = 0; k < 2; ++k)
    {
        const double* b = state + 5 * k;
        const double dm = rates[k];
        const double fx = rates[6 + 2 * k] + rates[2 + 2 * k];
        const double fy = rates[7 + 2 * k] + rates[3 + 2 * k];
        ds[5 * k + 0] = dm;
        ds[5 * k + 3] = (fx - b[3] * dm) / b[0];
        ds[5 * k + 4] = (fy - b[4] * dm) / b[0];
    }
    // step h: a relative change of about 1e-6 in the fastest-changing entry
    double rel = 0.0;
    for (int k = 0; k < 2; ++k)
    {
        const double* b = state + 5 * k;
        const double v = std::hypot(b[3], b[4]);
        rel = std::max(rel, std::fabs(ds[5 * k]) / b[0]);
        if (v > 0.0) rel = std::max(rel, std::hypot(ds[5 * k + 3], ds[5 * k + 4]) / v);
    }
    if (rel == 0.0)
    {
        for (int k = 0; k < 4; ++k) out[k] = 0.0;
        return MARA_OK;
    }
    const double h = 1e-6 / rel;
    double sp[10], sm[10], ep[10], em[10];
    for (int k = 0; k < 10; ++k)
    {
        sp[k] = state[k] + h * ds[k];
        sm[k] = state[k] - h * ds[k];
    }
    MARA_REQUIRE(elements(sp, time, ep) && elements(sm, time, em),
                 "mara_two_body_element_rates: the perturbed orbit is not bound");
    for (int k = 0; k < 4; ++k) out[k] = (ep[k] - em[k]) / (2.0 * h);
    return MARA_OK;
}

} // extern "C"
