// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// CPU restatement of the reference's spherical-track SRHD scheme
// (src/scheme_sedov2d.cpp, the moving radial tracks of problems/sedov2d.cpp),
// gamma = 4/3, temperature floor 1e-6:
//   cell_volume / face_area                 :40-62
//   recover_primitive                       :150-181  (u / dV, srhd recovery)
//   radial_gradient                         :188-203  (PLM on cell-centre radii, theta 1 or 0)
//   radial_godunov_data                     :208-230  (HLLC flux across the contact, contact speed)
//   sample                                  :235-253
//   polar_godunov_data                      :258-311  (transverse faces of two tracks, mesh_sliding.hpp:122-172)
//   delta_conserved / delta_face_positions  :316-356
// and the driver glue of problems/sedov2d.cpp:563-660 (boundary Riemann data
// from given ghost primitives, polar faces between neighbouring tracks,
// forward-Euler update) with the RK combinations of src/app_control.hpp:169-195.
// Arithmetic keeps the reference's evaluation order.
//
// Flat layout: T tracks; ncells[j] cells on track j; theta[2j], theta[2j+1];
// radii: concatenated face radii (ncells[j] + 1 per track); u: concatenated
// conserved volume integrals, 5 per cell (D, S1, S2, S3, tau).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "oracle_common.hpp"
#include "srhd_common.hpp"

namespace {

using namespace oracle::srhd;

const double kGamma = 4. / 3;
const double kFloor = 1e-6;

struct Track
{
    int64_t n;                 // cells
    double t0, t1;
    const double* r;           // n + 1 face radii
};

inline double cell_volume(double r0, double r1, double t0, double t1)
{
    double dcost = -(std::cos(t1) - std::cos(t0));
    return 2.0 * M_PI * (r1 * r1 * r1 - r0 * r0 * r0) / 3.0 * dcost;
}

inline double face_area(double r0, double r1, double t0, double t1)
{
    double R0 = r0 * std::sin(t0);
    double R1 = r1 * std::sin(t1);
    double z0 = r0 * std::cos(t0);
    double z1 = r1 * std::cos(t1);
    double dR = R1 - R0;
    double dz = z1 - z0;
    return M_PI * (R0 + R1) * std::pow(dR * dR + dz * dz, 0.5);
}

inline double center_theta(const Track& t) { return 0.5 * (t.t0 + t.t1); }
inline double center_radius(const Track& t, int64_t i) { return 0.5 * (t.r[i] + t.r[i + 1]); }

// plm_gradient_scalar_t on coordinates (scheme_plm_gradient.hpp:44-67)
inline double plm_x(double xl, double x0, double xr, double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) / (x0 - xl) * theta;
    double b = (yr - yl) / (xr - xl);
    double c = (yr - y0) / (xr - x0) * theta;
    double sa = std::copysign(1.0, a), sb = std::copysign(1.0, b), sc = std::copysign(1.0, c);
    return 0.25 * std::abs(sa + sb) * (sa + sc) * std::min(std::min(std::abs(a), std::abs(b)), std::abs(c));
}

struct TrackData
{
    const Track* t = nullptr;            // null: the empty track data beyond a pole
    const Prim* pc = nullptr;
    const Prim* dc = nullptr;
};

// sedov::sample (scheme_sedov2d.cpp:235-253)
Prim sample(const TrackData& d, double r, int64_t index, const Prim& fallback)
{
    const Track& t = *d.t;
    if (r <= t.r[0] || r >= t.r[t.n]) return fallback;
    index = std::min(index, t.n);
    while (r < t.r[index + 0]) --index;
    while (r > t.r[index + 1]) ++index;
    double rc = 0.5 * (t.r[index] + t.r[index + 1]);
    Prim out;
    for (int k = 0; k < 5; ++k) put(out, k, get(d.pc[index], k) + get(d.dc[index], k) * (r - rc));
    return out;
}

struct PolarFace { Cons f; double da; int64_t il, ir; bool valid; };

// sedov::polar_godunov_data (scheme_sedov2d.cpp:258-311) over the transverse
// faces of tracks t1 | t2 (mesh::transverse_faces, mesh_sliding.hpp:122-172)
int polar_faces(const TrackData& d0, const TrackData& d1, const TrackData& d2, const TrackData& d3, bool use_plm,
                std::vector<PolarFace>& out)
{
    const Track& L = *d1.t;
    const Track& R = *d2.t;
    const int64_t nl = L.n + 1, nr = R.n + 1;
    // merge_sort (mesh_sliding.hpp:64-92): L first on ties
    std::vector<std::pair<double, char>> m;
    for (int64_t a = 0, b = 0; a < nl || b < nr;)
    {
        if (a < nl && (b == nr || L.r[a] <= R.r[b])) m.push_back({L.r[a++], 'L'});
        else m.push_back({R.r[b++], 'R'});
    }
    out.assign(nl + nr - 1, PolarFace{});
    int64_t il = -1, ir = -1;
    int bad = 0;
    for (size_t n = 0; n + 1 < m.size(); ++n)
    {
        il += m[n].second == 'L';
        ir += m[n].second == 'R';
        PolarFace& pf = out[n];
        pf.il = il;
        pf.ir = ir;
        pf.valid = il >= 0 && il + 1 < nl && ir >= 0 && ir + 1 < nr;
        if (!pf.valid)
        {
            pf.f = Cons{};
            pf.da = 0.0;
            continue;
        }
        const double ri = m[n].first, ro = m[n + 1].first;
        const double ql = L.t1, qr = R.t0;
        const double rf = 0.5 * (ri + ro);
        Prim pl, pr;
        if (!use_plm || !d0.t || !d3.t)
        {
            pl = sample(d1, rf, il, Prim{});
            pr = sample(d2, rf, ir, Prim{});
        }
        else
        {
            const double q0 = center_theta(*d0.t), q1 = center_theta(L), q2 = center_theta(R), q3 = center_theta(*d3.t);
            Prim p1 = sample(d1, rf, il, Prim{});
            Prim p2 = sample(d2, rf, ir, Prim{});
            Prim p0 = sample(d0, rf, il, p1);
            Prim p3 = sample(d3, rf, ir, p2);
            Prim cl, cr;
            for (int k = 0; k < 5; ++k)
            {
                put(cl, k, plm_x(q0, q1, q2, get(p0, k), get(p1, k), get(p2, k), 1.0));
                put(cr, k, plm_x(q1, q2, q3, get(p1, k), get(p2, k), get(p3, k), 1.0));
            }
            for (int k = 0; k < 5; ++k)
            {
                put(pl, k, get(p1, k) + (ql - q1) * get(cl, k));
                put(pr, k, get(p2, k) + (qr - q2) * get(cr, k));
            }
        }
        bad += riemann(pl, pr, 2, kGamma, true, pf.f, HLLC_FIXED);
        pf.da = face_area(ri, ro, ql, qr);
    }
    return bad;
}

struct Set
{
    int T;
    std::vector<Track> tracks;
    std::vector<int64_t> co;       // cell offsets
};

Set make_set(int32_t T, const int64_t* ncells, const double* theta, const double* radii)
{
    Set s;
    s.T = T;
    s.co.assign(T + 1, 0);
    const double* r = radii;
    for (int j = 0; j < T; ++j)
    {
        s.tracks.push_back(Track{ncells[j], theta[2 * j], theta[2 * j + 1], r});
        r += ncells[j] + 1;
        s.co[j + 1] = s.co[j] + ncells[j];
    }
    return s;
}

// One forward-Euler advance (problems/sedov2d.cpp:608-660). Returns 0, or 1
// where the reference throws (a recovery or a contact speed failed).
int advance(const Set& S, const double* u, const double* ghost_in, const double* ghost_out, double dt, bool use_plm,
            double* radii_out, double* u_out, double* prim_out, double* grad_out, double* radial_out, double* polar_out)
{
    const int T = S.T;
    const int64_t C = S.co[T];
    std::vector<Prim> pc(C), dc(C);
    std::vector<Cons> ff(C + T);
    std::vector<double> vh(C + T);
    int bad = 0;
    for (int j = 0; j < T; ++j)
    {
        const Track& t = S.tracks[j];
        const int64_t c0 = S.co[j], f0 = S.co[j] + j;
        for (int64_t i = 0; i < t.n; ++i)
        {
            const double dv = cell_volume(t.r[i], t.r[i + 1], t.t0, t.t1);
            double z[5];
            for (int k = 0; k < 5; ++k) z[k] = u[5 * (c0 + i) + k] / dv;
            int it = 0;
            bad += recover_primitive(z, kGamma, kFloor, 0.0, pc[c0 + i], it) != 0;
        }
        // radial_gradient: interior cells, zeros at both ends
        for (int64_t i = 0; i < t.n; ++i)
        {
            Prim g{0, 0, 0, 0, 0};
            if (i > 0 && i + 1 < t.n)
            {
                const double xl = center_radius(t, i - 1), x0 = center_radius(t, i), xr = center_radius(t, i + 1);
                for (int k = 0; k < 5; ++k)
                    put(g, k, plm_x(xl, x0, xr, get(pc[c0 + i - 1], k), get(pc[c0 + i], k), get(pc[c0 + i + 1], k),
                                    use_plm ? 1.0 : 0.0));
            }
            dc[c0 + i] = g;
        }
        // radial_godunov_data with the driver's inner_bc / outer_bc
        {
            const Prim gi = load_prim(ghost_in + 5 * j);
            const Prim& front = pc[c0];
            const double vel = std::min(1.0 * front.u1 / lorentz_factor(front), 0.0);
            bad += riemann(gi, front, 1, kGamma, true, ff[f0], HLLC_MOVING_FACE, vel);
            vh[f0] = vel;
        }
        for (int64_t i = 1; i < t.n; ++i)
        {
            const double drl = t.r[i] - t.r[i - 1], drr = t.r[i + 1] - t.r[i];
            Prim pl, pr;
            for (int k = 0; k < 5; ++k)
            {
                put(pl, k, get(pc[c0 + i - 1], k) + 0.5 * get(dc[c0 + i - 1], k) * drl);
                put(pr, k, get(pc[c0 + i], k) - 0.5 * get(dc[c0 + i], k) * drr);
            }
            double as = 0.0;
            bad += riemann(pl, pr, 1, kGamma, true, ff[f0 + i], HLLC_ACROSS_CONTACT, 0.0, &as);
            vh[f0 + i] = as;
        }
        {
            const Prim go = load_prim(ghost_out + 5 * j);
            const double vel = 1.0 * go.u1 / lorentz_factor(go);
            bad += riemann(pc[c0 + t.n - 1], go, 1, kGamma, true, ff[f0 + t.n], HLLC_MOVING_FACE, vel);
            vh[f0 + t.n] = vel;
        }
    }
    // polar faces of every interface j | j + 1
    std::vector<std::vector<PolarFace>> gf(T + 1);
    auto td = [&] (int j) {
        TrackData d;
        if (j >= 0 && j < T) { d.t = &S.tracks[j]; d.pc = &pc[S.co[j]]; d.dc = &dc[S.co[j]]; }
        return d;
    };
    for (int j = 0; j + 1 < T; ++j) bad += polar_faces(td(j - 1), td(j), td(j + 1), td(j + 2), use_plm, gf[j + 1]);

    // delta_conserved + delta_face_positions
    for (int j = 0; j < T; ++j)
    {
        const Track& t = S.tracks[j];
        const int64_t c0 = S.co[j], f0 = S.co[j] + j;
        std::vector<Cons> gl(t.n, Cons{}), gr(t.n, Cons{});
        for (const PolarFace& p : gf[j])        // this track is the right side: bin by ir
        {
            const int64_t b = p.valid ? p.ir : 0;
            for (int k = 0; k < 5; ++k) gl[b].c[k] = gl[b].c[k] + p.f.c[k] * p.da;
        }
        for (const PolarFace& p : gf[j + 1])    // the left side: bin by il
        {
            const int64_t b = p.valid ? p.il : 0;
            for (int k = 0; k < 5; ++k) gr[b].c[k] = gr[b].c[k] + p.f.c[k] * p.da;
        }
        const double qc = center_theta(t);
        for (int64_t i = 0; i < t.n; ++i)
        {
            const double da0 = face_area(t.r[i], t.r[i], t.t0, t.t1);
            const double da1 = face_area(t.r[i + 1], t.r[i + 1], t.t0, t.t1);
            const double dv = cell_volume(t.r[i], t.r[i + 1], t.t0, t.t1);
            const Prim& p = pc[c0 + i];
            const double rc = center_radius(t, i);
            // spherical_geometry_source_terms (physics_srhd.hpp:330-345)
            const double cotq = std::tan(M_PI_2 - qc);
            const double ur = p.u1, uq = p.u2, up = p.u3, pg = p.p;
            const double H0 = enthalpy_density(p, kGamma);
            const double src[5] = {0.0 / 1.0, (2.0 * pg + H0 * (uq * uq + up * up)) / rc,
                                   (cotq * pg + H0 * (up * up * cotq - ur * uq)) / rc,
                                   -up * H0 * (ur + uq * cotq) / rc, 0.0 / 1.0};
            for (int k = 0; k < 5; ++k)
            {
                const double df = ff[f0 + i + 1].c[k] * da1 - ff[f0 + i].c[k] * da0;
                const double dg = gr[i].c[k] - gl[i].c[k];
                const double sc = src[k] * dv;
                u_out[5 * (c0 + i) + k] = u[5 * (c0 + i) + k] + (-(df + dg) + sc) * dt;
            }
            if (prim_out)
                for (int k = 0; k < 5; ++k) prim_out[5 * (c0 + i) + k] = get(p, k);
            if (grad_out)
                for (int k = 0; k < 5; ++k) grad_out[5 * (c0 + i) + k] = get(dc[c0 + i], k);
        }
        for (int64_t i = 0; i <= t.n; ++i)
        {
            radii_out[f0 + i] = t.r[i] + vh[f0 + i] * dt;
            if (radial_out)
            {
                for (int k = 0; k < 5; ++k) radial_out[6 * (f0 + i) + k] = ff[f0 + i].c[k];
                radial_out[6 * (f0 + i) + 5] = vh[f0 + i];
            }
        }
    }
    if (polar_out)
        for (int j = 0; j + 1 < T; ++j)
            for (const PolarFace& p : gf[j + 1])
            {
                for (int k = 0; k < 5; ++k) *polar_out++ = p.f.c[k];
                *polar_out++ = p.da;
                *polar_out++ = p.valid ? double(p.il) : 0.0;
                *polar_out++ = p.valid ? double(p.ir) : 0.0;
            }
    return bad ? 1 : 0;
}

} // namespace

extern "C" {

// One forward-Euler advance of every track (see the header for the layout);
// the optional outputs follow ref_sedov_advance. Returns 1 on a failure the
// reference throws for.
int oracle_sedov_advance(int32_t T, const int64_t* ncells, const double* theta, const double* radii, const double* u,
                         const double* ghost_in, const double* ghost_out, double dt, int32_t use_plm,
                         double* radii_out, double* u_out, double* prim, double* grad, double* radial, double* polar)
{
    const Set S = make_set(T, ncells, theta, radii);
    return advance(S, u, ghost_in, ghost_out, dt, use_plm != 0, radii_out, u_out, prim, grad, radial, polar);
}

// control::advance_runge_kutta (app_control.hpp:169-195) of the advance,
// radii and conserved combined by weighted_sum (problems/sedov2d.cpp:127-152);
// ghost_in / ghost_out hold rk_order stages of 5 T primitives (the boundary
// states of each stage). In place on radii and u.
int oracle_sedov_advance_rk(int32_t T, const int64_t* ncells, const double* theta, double* radii, double* u,
                            const double* ghost_in, const double* ghost_out, double dt, int32_t rk_order,
                            int32_t use_plm)
{
    int64_t C = 0;
    for (int j = 0; j < T; ++j) C += ncells[j];
    const int64_t F = C + T;
    std::vector<double> r0(radii, radii + F), u0(u, u + 5 * C), r1(F), u1(5 * C), r2(F), u2(5 * C);
    auto step = [&] (const double* rin, const double* uin, int stage, double* rout, double* uout) {
        const Set S = make_set(T, ncells, theta, rin);
        return advance(S, uin, ghost_in + 5 * T * stage, ghost_out + 5 * T * stage, dt, use_plm != 0, rout, uout,
                       nullptr, nullptr, nullptr, nullptr);
    };
    // weighted_sum(s, t, b) = s b + t (1 - b), into t
    auto mix = [&] (double b, double b1, const double* rs, const double* us, double* rt, double* ut) {
        for (int64_t k = 0; k < F; ++k) rt[k] = rs[k] * b + rt[k] * b1;
        for (int64_t k = 0; k < 5 * C; ++k) ut[k] = us[k] * b + ut[k] * b1;
    };
    int bad = 0;
    if (rk_order == 1) return step(r0.data(), u0.data(), 0, radii, u);
    bad |= step(r0.data(), u0.data(), 0, r1.data(), u1.data());
    bad |= step(r1.data(), u1.data(), 1, r2.data(), u2.data());
    if (rk_order == 2)
    {
        mix(1.0 / 2, 1.0 / 2, r0.data(), u0.data(), r2.data(), u2.data());
    }
    else
    {
        mix(3.0 / 4, 1.0 / 4, r0.data(), u0.data(), r2.data(), u2.data());
        bad |= step(r2.data(), u2.data(), 2, r1.data(), u1.data());
        mix(1.0 / 3, 2.0 / 3, r0.data(), u0.data(), r1.data(), u1.data());
        r2 = r1;
        u2 = u1;
    }
    std::memcpy(radii, r2.data(), F * sizeof(double));
    std::memcpy(u, u2.data(), 5 * C * sizeof(double));
    return bad;
}

// sedov::remesh (scheme_sedov2d.cpp:362-412) of one track, in place on
// radii (capacity ncells + 2) and u (capacity 5 (ncells + 1)): drop the
// first cell while the inner face lies inside inner_radius, split the cell
// of largest aspect dr / (r_c dtheta) if above the maximum (and stop), merge
// the cell of smallest aspect with its smaller-aspect neighbour if below the
// minimum. The reference recurses after a drop or a merge with the two
// aspect bounds passed in swapped order (make_track calls remesh(..., min,
// max, ...) into parameters (max, min)), so each further level runs with
// the bounds exchanged; that is restated. Returns the new cell count, or -1
// where the reference throws (a merge on a one-cell track).
int64_t oracle_sedov_remesh(int64_t ncells, double theta0, double theta1, double* radii, double* u,
                            double max_aspect, double min_aspect, double inner_radius)
{
    std::vector<double> rf(radii, radii + ncells + 1), uc(u, u + 5 * ncells);
    double amax_bound = max_aspect, amin_bound = min_aspect;
    for (;;)
    {
        const int64_t n = int64_t(rf.size()) - 1;
        if (n < 1) return -1;
        std::vector<double> aspect(n);
        for (int64_t i = 0; i < n; ++i)
        {
            const double dr = rf[i + 1] - rf[i];
            const double rc = 0.5 * (rf[i] + rf[i + 1]);
            aspect[i] = dr / (rc * (theta1 - theta0));
        }
        // nd::argmin / argmax: the first index holding the min / max
        const double mn = *std::min_element(aspect.begin(), aspect.end());
        const double mx = *std::max_element(aspect.begin(), aspect.end());
        int64_t imin = 0, imax = 0;
        while (!(aspect[imin] == mn)) ++imin;
        while (!(aspect[imax] == mx)) ++imax;
        auto remove = [&] (int64_t e) -> bool {
            if (e == 0 || e + 1 >= int64_t(rf.size())) return false;
            rf.erase(rf.begin() + e);
            for (int k = 0; k < 5; ++k) uc[5 * (e - 1) + k] = uc[5 * (e - 1) + k] + uc[5 * e + k];
            uc.erase(uc.begin() + 5 * e, uc.begin() + 5 * e + 5);
            return true;
        };
        if (rf.front() < inner_radius)
        {
            if (n < 2) return -1;   // the reference would drop into an empty track
            rf.erase(rf.begin());
            uc.erase(uc.begin(), uc.begin() + 5);
            std::swap(amax_bound, amin_bound);
            continue;
        }
        if (aspect[imax] > amax_bound)
        {
            const double mid = 0.5 * (rf[imax] + rf[imax + 1]);
            rf.insert(rf.begin() + imax + 1, mid);
            double half[5];
            for (int k = 0; k < 5; ++k) half[k] = 0.5 * uc[5 * imax + k];
            for (int k = 0; k < 5; ++k) uc[5 * imax + k] = half[k];
            uc.insert(uc.begin() + 5 * (imax + 1), half, half + 5);
            break;
        }
        if (aspect[imin] < amin_bound)
        {
            int64_t e = -1;
            if (imin == 0) e = 1;
            else if (imin + 1 == n) e = imin;
            else if (aspect[imin - 1] <= aspect[imin + 1]) e = imin;
            else if (aspect[imin - 1] >= aspect[imin + 1]) e = imin + 1;
            if (e < 0) break;
            if (!remove(e)) return -1;
            std::swap(amax_bound, amin_bound);
            continue;
        }
        break;
    }
    std::copy(rf.begin(), rf.end(), radii);
    std::copy(uc.begin(), uc.end(), u);
    return int64_t(rf.size()) - 1;
}

// sedov::cell_volume / face_area
double oracle_sedov_cell_volume(double r0, double r1, double t0, double t1) { return cell_volume(r0, r1, t0, t1); }
double oracle_sedov_face_area(double r0, double r1, double t0, double t1) { return face_area(r0, r1, t0, t1); }

} // extern "C"
