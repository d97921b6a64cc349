/* C entry point to the reference's calc_na_val (na_calc.cpp:308-327),
 * compiled from the reference's own source by build_ref.sh. */
#include <tuple>
#include <vector>

double calc_na_val(std::vector<std::tuple<double, double>> points, std::vector<std::tuple<double, double>> disps,
                   double minx, double miny, double axial_strain, double shear_strain);

extern "C" double ref_calc_na_val(int n, const double *xy, const double *uv, double minx, double miny,
                                  double axial_strain, double shear_strain) {
    std::vector<std::tuple<double, double>> p(n), u(n);
    for (int i = 0; i < n; ++i) {
        p[i] = std::make_tuple(xy[2 * i], xy[2 * i + 1]);
        u[i] = std::make_tuple(uv[2 * i], uv[2 * i + 1]);
    }
    return calc_na_val(p, u, minx, miny, axial_strain, shear_strain);
}
