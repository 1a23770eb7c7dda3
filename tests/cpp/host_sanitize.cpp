// Every host-side entry point of the propagator library and the oracle, for a build with
// -fsanitize=address,undefined: parameter blocks, Earth models (valid and invalid),
// trajectories over the whole cosine range including shell-grazing ones, production-height
// shifts, model files (2, 3 and 5 columns, comments, malformed), and oracle atmospheric,
// averaged and beam runs.  Prints "ok" when every check passed.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "cp3_host.hpp"
#include "../../oracle/cp3_oracle.h"

using namespace cp3;

static int failures = 0;
#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::printf("check failed at line %d: %s\n", __LINE__, #c);   \
            failures++;                                                   \
        }                                                                 \
    } while (0)

static std::string write_file(const char* name, const char* text) {
    std::string path = std::string(std::getenv("SANITIZE_TMP") ? std::getenv("SANITIZE_TMP") : "/tmp") + "/" + name;
    FILE* f = std::fopen(path.c_str(), "w");
    std::fputs(text, f);
    std::fclose(f);
    return path;
}

int main() {
    // parameter blocks: both orderings, both neutrino types, degenerate splittings
    for (double dm23 : {2.49e-3, -2.49e-3, 0.0})
        for (double dm12 : {7.53e-5, 0.0})
            for (int anti = 0; anti < 2; anti++) {
                MixingInput m;
                m.theta12 = 0.5843; m.theta13 = 0.1496; m.theta23 = 0.7365; m.dcp = -1.601;
                m.knutype = anti ? -1 : 1; m.dm12sq = dm12; m.dm23sq = dm23;
                OscParams p;
                build_osc_params(m, anti, &p);
                CHECK(std::isfinite(p.h0[0]) && std::isfinite(p.cpoly[2]));
            }

    // Earth models
    const double r[5] = {0.0, 1220.0, 3480.0, 5701.0, 6371.0};
    const double rho[5] = {13.0, 13.0, 11.3, 5.0, 3.3};
    const double ye[5] = {0.468, 0.468, 0.468, 0.497, 0.497};
    // the quadratic model of PREM_4layer_quad_v2 (density a r^2 + b r + c, r in km)
    const double rq[5] = {0.0, 1221.5, 3480.0, 5701.0, 6371.0};
    const double a[5] = {-2.1779e-07, -2.1779e-07, -2.46861e-07, -3.0796e-08, -1.72335e-06},
                 b[5] = {0.0, 0.0, 0.000171088, -0.00024486, 0.019358},
                 c[5] = {13.09, 13.09, 12.31, 6.78, -50.42};
    EarthModel e, ep;
    std::string err;
    CHECK(make_earth_model(r, rho, nullptr, nullptr, ye, 5, false, &e, &err) == 0);
    CHECK(make_earth_model(rq, a, b, c, ye, 5, true, &ep, &err) == 0);
    const double bad_r[3] = {0.0, 3480.0, 1220.0};
    EarthModel bad;
    CHECK(make_earth_model(bad_r, rho, nullptr, nullptr, ye, 3, false, &bad, &err) != 0);
    CHECK(make_earth_model(r, rho, nullptr, nullptr, ye, 0, false, &bad, &err) != 0);

    // trajectories: a fine sweep, the shell-grazing cosines and both ends
    std::vector<double> cz;
    for (int i = 0; i <= 400; i++) cz.push_back(-1.0 + 2.0 * i / 400);
    for (int i = 1; i < 5; i++) cz.push_back(-std::sqrt(1.0 - r[i] * r[i] / (6371.0 * 6371.0)));
    for (const EarthModel* em : {&e, &ep})
        for (double h_km : {0.0, 22.0, 100.0}) {
            TrajectoryTable t;
            CHECK(build_trajectories(*em, cz.data(), (int)cz.size(), h_km * 1e5, &t, &err) == 0);
            CHECK((int)t.offset.size() == (int)cz.size() + 1);
            for (size_t i = 0; i < t.len_km.size(); i++)
                if (!(t.len_km[i] >= -1e-6)) {
                    std::printf("segment %zu length %.17g (h %g km)\n", i, t.len_km[i], h_km);
                    failures++;
                }
        }
    for (double x : cz) CHECK(count_shells(e, x) >= 0);

    // production-height shifts
    const double edges[6] = {8.0, 12.0, 17.0, 24.0, 33.0, 45.0};
    std::vector<double> shifts;
    production_height_shifts(cz.data(), (int)cz.size(), 20e5, edges, 5, &shifts);
    CHECK(shifts.size() == cz.size() * 6);

    // model files
    int ncols = 0;
    std::vector<std::vector<double>> cols;
    const std::string f3 = write_file("m3.dat", "# r rho ye\n0 13 0.468\n1220 13 0.468\n3480 11.3 0.468\n\n5701 5 0.497\n6371 3.3 0.497\n");
    CHECK(parse_model_file(f3.c_str(), &ncols, &cols, &err) == 0 && ncols == 3 && cols[0].size() == 5);
    const std::string f2 = write_file("m2.dat", "0 13\n1220 13\n3480 11.3\n6371 3.3\n");
    CHECK(parse_model_file(f2.c_str(), &ncols, &cols, &err) == 0 && ncols == 2);
    const std::string f5 = write_file("m5.dat", "0 13 0 -8.8 0.468\n1220 13 0 -8.8 0.468\n6371 5.3 -0.5 0 0.497\n");
    CHECK(parse_model_file(f5.c_str(), &ncols, &cols, &err) == 0 && ncols == 5);
    const std::string fb = write_file("bad.dat", "0 13 0.468\n1220 abc 0.468\n");
    CHECK(parse_model_file(fb.c_str(), &ncols, &cols, &err) != 0);
    const std::string fm = write_file("mixed.dat", "0 13 0.468\n1220 13\n");
    CHECK(parse_model_file(fm.c_str(), &ncols, &cols, &err) != 0);
    CHECK(parse_model_file("/nonexistent/model.dat", &ncols, &cols, &err) != 0);

    // the oracle: atmospheric (constant and quadratic), averaged, beam
    orc_mixing mix{0.5843, 0.1496, 0.7365, -1.601, 1, 7.53e-5, 2.49e-3};
    // the oracle takes the reference's internal order: radii descending, r = 0 row last
    double rd[5], rqd[5], rhod[5], yed[5], ad[5], bd[5], cd[5], yq[5];
    CHECK(orc_flip_model(5, r, rho, ye, nullptr, nullptr, rd, rhod, yed, nullptr, nullptr) == 0);
    CHECK(orc_flip_model(5, rq, a, b, c, ye, rqd, ad, bd, cd, yq) == 0);
    orc_earth oe{5, rd, rhod, yed, nullptr, nullptr, nullptr, 0};
    orc_earth oq{5, rqd, nullptr, yq, ad, bd, cd, 1};
    std::vector<double> en;
    for (int i = 0; i < 17; i++) en.push_back(std::pow(10.0, -1.0 + 3.0 * i / 16));
    const int nc = (int)cz.size(), ne = (int)en.size(), nb = 5;
    std::vector<double> out((size_t)nc * ne * 9), ph((size_t)2 * 3 * ne * nc * nb, 1.0 / nb);
    for (const orc_earth* oem : {&oe, &oq}) {
        CHECK(orc_atmos(&mix, 0, cz.data(), nc, en.data(), ne, oem, 22.0, 0, 0, nullptr, nullptr,
                        64, 1, out.data()) == 0);
        double worst = 0.0;
        int wic = 0, wie = 0;
        for (int ic = 0; ic < nc; ic++)
            for (int ie = 0; ie < ne; ie++) {
                double s = 0.0;
                for (int k = 0; k < 3; k++) s += out[((size_t)ic * ne + ie) * 9 + k];
                if (std::fabs(s - 1.0) > worst) {
                    worst = std::fabs(s - 1.0);
                    wic = ic;
                    wie = ie;
                }
            }
        if (!(worst < 1e-10)) {  // unitarity: sum over final flavours
            std::printf("unitarity %.3e at cos %.6f E %.4f (poly %d)\n", worst, cz[wic], en[wie], oem->poly);
            failures++;
        }
        CHECK(orc_atmos(&mix, 1, cz.data(), nc, en.data(), ne, oem, 20.0, 1, nb, ph.data(), edges,
                        64, 1, out.data()) == 0);
    }
    std::vector<double> eb(1000), ob(1000 * 9);
    for (int i = 0; i < 1000; i++) eb[i] = 0.1 + 9.9 * i / 999;
    CHECK(orc_beam(&mix, 0, eb.data(), 1000, 2.6, 1300.0, 1, ob.data()) == 0);
    double A[18];
    orc_transition_matrix(&mix, 0, 1.0, 1.3, 810.0, A);
    CHECK(std::isfinite(A[0]));

    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
