// cp3_host.cpp -- host side of the propagator (no CUDA).  The formulas that feed FP64
// parity (mixing matrix, mass matrix, root order, segment geometry and densities) keep the
// reference's evaluation order so that the device sees bit-identical inputs.
#include "cp3_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "../../include/cudaprob3_gb300.h"

namespace cp3 {

void build_osc_params(const MixingInput& m, int antineutrino, OscParams* o) {
    std::memset(o, 0, sizeof(*o));
    // setMNSMatrix (propagator.hpp:148-183)
    double dcp = m.dcp;
    if (m.knutype < 0) dcp *= -1;
    const double s12 = std::sin(m.theta12), s13 = std::sin(m.theta13), s23 = std::sin(m.theta23);
    const double c12 = std::cos(m.theta12), c13 = std::cos(m.theta13), c23 = std::cos(m.theta23);
    const double sd = std::sin(dcp), cd = std::cos(dcp);
    double* U = o->U;
    auto set = [U](int i, int j, double re, double im) {
        U[(i * 3 + j) * 2] = re;
        U[(i * 3 + j) * 2 + 1] = im;
    };
    set(0, 0, c12 * c13, 0.0);
    set(0, 1, s12 * c13, 0.0);
    set(0, 2, s13 * cd, -s13 * sd);
    set(1, 0, -s12 * c23 - c12 * s23 * s13 * cd, -c12 * s23 * s13 * sd);
    set(1, 1, c12 * c23 - s12 * s23 * s13 * cd, -s12 * s23 * s13 * sd);
    set(1, 2, s23 * c13, 0.0);
    set(2, 0, s12 * s23 - c12 * c23 * s13 * cd, -c12 * c23 * s13 * sd);
    set(2, 1, -c12 * s23 - s12 * c23 * s13 * cd, -s12 * c23 * s13 * sd);
    set(2, 2, c23 * c13, 0.0);

    // setNeutrinoMasses (propagator.hpp:188-209)
    double mv[3] = {0.0, m.dm12sq, m.dm12sq + m.dm23sq};
    const double delta = 5.0e-9;
    if (m.dm12sq == 0.0) mv[0] -= delta;
    if (m.dm23sq == 0.0) mv[2] += delta;
    double* D = o->dm;
    D[0] = D[4] = D[8] = 0.0;
    D[1] = mv[0] - mv[1];
    D[3] = -D[1];
    D[2] = mv[0] - mv[2];
    D[6] = -D[2];
    D[5] = mv[1] - mv[2];
    D[7] = -D[5];

    // prepare_getMfast (physics.hpp:198-252): vacuum roots, then which root is which state.
    {
        const double aV = D[1] + D[2];
        const double bV = D[1] * D[2];
        const double gV = 0.0;
        double t = aV * aV - 3.0 * bV;
        double arg = (2.0 * aV * aV * aV - 9.0 * aV * bV + 27.0 * gV) / (2.0 * std::sqrt(t * t * t));
        if (std::fabs(arg) > 1.0) arg = arg / std::fabs(arg);
        const double th0 = std::acos(arg) / 3.0;
        const double th1 = th0 - (2.0 * M_PI / 3.0);
        const double th2 = th0 + (2.0 * M_PI / 3.0);
        double r[3];
        r[0] = r[1] = r[2] = -(2.0 / 3.0) * std::sqrt(t);
        r[0] *= std::cos(th0);
        r[1] *= std::cos(th1);
        r[2] *= std::cos(th2);
        t = D[0] - aV / 3.0;
        for (double& x : r) x += t;
        for (int i = 0; i < 3; i++) {
            double best = std::fabs(D[i * 3] - r[0]);
            int k = 0;
            for (int j = 1; j < 3; j++) {
                const double d = std::fabs(D[i * 3] - r[j]);
                if (d < best) {
                    k = j;
                    best = d;
                }
            }
            o->order[i] = k;
        }
    }

    // Rotated real basis: O = R13 R12, H0 = O diag(DM(k,0)) O^T.
    const double O[3][3] = {{c13 * c12, c13 * s12, s13}, {-s12, c12, 0.0}, {-s13 * c12, -s13 * s12, c13}};
    const double dk[3] = {D[0], D[3], D[6]};
    const int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    for (int q = 0; q < 6; q++) {
        const int i = ij[q][0], j = ij[q][1];
        o->h0[q] = O[i][0] * O[j][0] * dk[0] + O[i][1] * O[j][1] * dk[1] + O[i][2] * O[j][2] * dk[2];
    }
    const double* h = o->h0;
    o->cpoly[0] = h[0] + h[3] + h[5];
    o->cpoly[1] = h[0] * h[3] - h[1] * h[1] + h[0] * h[5] - h[2] * h[2] + h[3] * h[5] - h[4] * h[4];
    o->cpoly[2] = h[0] * (h[3] * h[5] - h[4] * h[4]) - h[1] * (h[1] * h[5] - h[4] * h[2]) +
                  h[2] * (h[1] * h[4] - h[3] * h[2]);
    o->cpoly[3] = h[3] + h[5];
    o->cpoly[4] = h[3] * h[5] - h[4] * h[4];
    auto split = [](double x, float out[2]) {
        out[0] = (float)x;
        out[1] = (float)(x - (double)out[0]);
    };
    for (int q = 0; q < 5; q++) split(o->cpoly[q], o->cpolyf[q]);
    for (int k = 0; k < 3; k++) split(dk[k], o->muf[k]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            float hl[2];
            split(O[i][j], hl);
            o->of[i][j] = hl[0];
            o->oflo[i][j] = hl[1];
        }
    o->w[0] = c23;
    o->w[1] = s23;
    o->w[2] = cd;
    o->w[3] = sd;
    for (int k = 0; k < 4; k++) o->wf[k] = (float)o->w[k];
    o->anti = antineutrino ? 1 : 0;
}

int make_earth_model(const double* radii, const double* c1, const double* c2, const double* c3,
                     const double* ye, int n, bool poly, EarthModel* out, std::string* err) {
    if (n <= 0 || !radii || !c1 || !ye || (poly && (!c2 || !c3))) {
        *err = "setDensity : vectors must not be empty";
        return CP3_ERR_BAD_SIZE;
    }
    bool flip = false;
    if (n >= 2) {
        const int sign = radii[1] - radii[0] > 0 ? 1 : -1;
        for (int i = 1; i < n; i++)
            if ((radii[i] - radii[i - 1]) * sign < 0) {
                *err = "radii order messed up";
                return CP3_ERR_ORDER;
            }
        flip = sign == 1;
    }
    EarthModel e;
    e.poly = poly;
    auto take = [&](const double* src, std::vector<double>& dst) {
        dst.resize(n);
        for (int i = 0; i < n; i++) dst[i] = src[flip ? n - 1 - i : i];
    };
    take(radii, e.radii);
    take(ye, e.ye);
    if (poly) {
        take(c1, e.a);
        take(c2, e.b);
        take(c3, e.c);
    } else {
        take(c1, e.rho);
    }
    e.coslimit.resize(n);
    for (int i = 0; i < n; i++) {
        double x = -1 * std::sqrt(1 - (e.radii[i] * e.radii[i] / (kREarthKm * kREarthKm)));
        if (i == 0) x = 0;
        e.coslimit[i] = x;
    }
    *out = std::move(e);
    return CP3_OK;
}

int count_shells(const EarthModel& e, double c) {
    return (int)std::count_if(e.coslimit.begin(), e.coslimit.end(),
                              [c](double limit) { return c < limit; });
}

namespace {

// getTraversedDistanceOfLayer (physics.hpp:745-787), cm.  For the innermost crossed shell
// only its own radius is read.
double segment_cm(const EarthModel& e, int layer, int maxl, double path_cm, double earth_cm,
                  double cosz) {
    if (cosz >= 0) return path_cm;
    if (layer == 0) return path_cm - earth_cm;
    const int i = layer <= maxl ? layer - 1 : 2 * maxl - layer - 1;
    const double R2min = kREarthKm * kREarthKm * (1 - cosz * cosz);
    double cross_this = 2.0 * std::sqrt(e.radii[i] * e.radii[i] - R2min);
    if (std::sqrt(R2min) > e.radii[i]) cross_this = 0;
    if (i < maxl - 1) {
        double cross_next = 2.0 * std::sqrt(e.radii[i + 1] * e.radii[i + 1] - R2min);
        if (std::sqrt(R2min) > e.radii[i + 1]) cross_next = 0;
        return 0.5 * (cross_this - cross_next) * kKm2Cm;
    }
    return cross_this * kKm2Cm;
}

// getDensityOfLayerPoly (physics.hpp:651-739): mean of a r^2 + b r + c along the segment
// (parametrised from the shell's outer edge), times Ye.
double segment_density_poly(const EarthModel& e, double cosz, int layer, int maxl, double seg_cm) {
    if (cosz >= 0) return 0;
    if (layer == 0) return 0;
    const int i = layer <= maxl ? layer - 1 : 2 * maxl - layer - 1;
    const std::vector<double>& r = e.radii;
    const double Rmin2 = std::pow(kREarthKm, 2) * (1 - std::pow(cosz, 2));
    const double Rmax2 = std::pow(r[i], 2);
    const double half = std::sqrt(Rmax2 - Rmin2);
    if (Rmin2 == 0) {
        const double r_in = (size_t)i + 1 < r.size() ? r[i + 1] : 0.0;
        const double hi = e.a[i] * std::pow(r[i], 3) / 3. + e.b[i] * std::pow(r[i], 2) / 2. + e.c[i] * r[i];
        const double lo = e.a[i] * std::pow(r_in, 3) / 3. + e.b[i] * std::pow(r_in, 2) / 2. + e.c[i] * r_in;
        double density = hi - lo;
        density /= (r[i] - r_in);
        return density * e.ye[i];
    }
    const double qa = 1.0, qb = -2 * half, qc = Rmax2;
    const double t2 = seg_cm / kKm2Cm, t1 = 0.;
    const double sq = (qa * std::pow(t2, 3) / 3. + qb * std::pow(t2, 2) / 2. + qc * t2) -
                      (qa * std::pow(t1, 3) / 3. + qb * std::pow(t1, 2) / 2. + qc * t1);
    auto root = [&](double t) { return std::sqrt(qc + t * (qb + qa * t)); };
    const double p1 = (qb + 2. * qa * t2) * root(t2) / (4. * qa);
    const double m1 = (qb + 2. * qa * t1) * root(t1) / (4. * qa);
    const double disc = qb * qb - 4. * qa * qc;
    const double p2 = disc * std::log(qb + 2. * qa * t2 + 2. * std::sqrt(qa) * root(t2)) / (8. * std::pow(qa, 3. / 2.));
    const double m2 = disc * std::log(qb + 2. * qa * t1 + 2. * std::sqrt(qa) * root(t1)) / (8. * std::pow(qa, 3. / 2.));
    const double lin = (p1 - p2) - (m1 - m2);
    const double con = t2 - t1;
    const double density = (e.a[i] * sq + e.b[i] * lin + e.c[i] * con) / (t2 - t1);
    return density * e.ye[i];
}

}  // namespace

int build_trajectories(const EarthModel& e, const double* cosines, int nc, double height_cm,
                       TrajectoryTable* out, std::string* err) {
    TrajectoryTable t;
    t.offset.resize(nc + 1);
    t.maxlayers.resize(nc);
    t.offset[0] = 0;
    for (int ic = 0; ic < nc; ic++) {
        const int M = count_shells(e, cosines[ic]);
        if (M > kMaxShells) {
            *err = "setMaxlayers : invalid number of maxLayer";
            return CP3_ERR_LAYER_LIMIT;
        }
        t.maxlayers[ic] = M;
        t.offset[ic + 1] = t.offset[ic] + M + 1;
        t.max_segments = std::max(t.max_segments, M + 1);
    }
    const int total = t.offset[nc];
    t.air_cm.resize(nc);
    t.path_cm.resize(nc);
    t.len_km.resize(total);
    t.rho_e.resize(total);
    t.cls.resize(total);
    for (int ic = 0; ic < nc; ic++) {
        const double cosz = cosines[ic];
        const int M = t.maxlayers[ic];
        // calculate_atmos: TotalEarthLength (physics.hpp:837), PathLength (:897-898)
        const double earth_cm = -2.0 * cosz * kREarthCm;
        const double path_cm =
            std::sqrt((kREarthCm + height_cm) * (kREarthCm + height_cm) -
                      (kREarthCm * kREarthCm) * (1 - cosz * cosz)) -
            kREarthCm * cosz;
        t.path_cm[ic] = path_cm;
        for (int l = 0; l <= M; l++) {
            const int s = t.offset[ic] + l;
            const double d = segment_cm(e, l, M, path_cm, earth_cm, cosz);
            if (l == 0) t.air_cm[ic] = d;
            t.len_km[s] = d / kKm2Cm;
            if (e.poly) {
                t.rho_e[s] = segment_density_poly(e, cosz, l, M, d);
                t.cls[s] = -1;
            } else {
                // getDensityOfLayer (physics.hpp:634-646); l <= M so the index is l-1
                t.rho_e[s] = l == 0 ? 0.0 : e.rho[l - 1] * e.ye[l - 1];
                t.cls[s] = l;  // class l: air for l == 0, shell l-1 otherwise
            }
        }
    }
    *out = std::move(t);
    return CP3_OK;
}

void production_height_shifts(const double* cosines, int nc, double height_cm,
                              const double* edges_km, int nb, std::vector<double>* out) {
    out->assign((size_t)nc * (nb + 1), 0.0);
    const double R = kREarthCm;
    for (int ic = 0; ic < nc; ic++) {
        const double c = cosines[ic];
        const double path = std::sqrt((R + height_cm) * (R + height_cm) - (R * R) * (1 - c * c)) - R * c;
        for (int p = 0; p <= nb; p++) {
            const double hcm = kKm2Cm * edges_km[p];
            const double v = std::sqrt((R + hcm) * (R + hcm) - (R * R) * (1 - c * c)) - R * c;
            (*out)[(size_t)ic * (nb + 1) + p] = v - path;
        }
    }
}

int parse_model_file(const char* path, int* ncols, std::vector<std::vector<double>>* cols,
                     std::string* err) {
    std::ifstream f(path);
    if (!f) {
        *err = std::string("could not open density file ") + path;
        return CP3_ERR_FILE;
    }
    std::string line;
    int n = 0;
    std::vector<std::vector<double>> c;
    int lineno = 0;
    while (std::getline(f, line)) {
        lineno++;
        const size_t first = line.find_first_not_of(" \t\r");
        if (first == std::string::npos || line[first] == '#') continue;
        std::istringstream ss(line);
        std::vector<double> row;
        std::string tok;
        while (ss >> tok) {
            if (tok[0] == '#') break;
            char* end = nullptr;
            const double v = std::strtod(tok.c_str(), &end);
            if (end == tok.c_str() || *end != '\0') {
                *err = std::string("density file ") + path + ": not a number on line " + std::to_string(lineno);
                return CP3_ERR_FILE;
            }
            row.push_back(v);
        }
        if (row.empty()) continue;
        if (n == 0) {
            n = (int)row.size();
            if (n != 2 && n != 3 && n != 5) {
                *err = std::string("Unsupported earth model in ") + path + ": " + std::to_string(n) + " entries per line";
                return CP3_ERR_FILE;
            }
            c.assign(n, {});
        } else if ((int)row.size() != n) {
            *err = std::string("density file ") + path + ": inconsistent number of entries on line " + std::to_string(lineno);
            return CP3_ERR_FILE;
        }
        for (int k = 0; k < n; k++) c[k].push_back(row[k]);
    }
    if (n == 0) {
        *err = std::string("density file ") + path + " holds no rows";
        return CP3_ERR_FILE;
    }
    *ncols = n;
    *cols = std::move(c);
    return CP3_OK;
}

}  // namespace cp3
