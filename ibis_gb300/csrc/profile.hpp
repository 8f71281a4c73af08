// Boundary-layer inflow profile (BoundaryLayerProfile, boundary.cpp:48-94):
// natural cubic splines of the streamwise velocity and the temperature over the
// wall-normal coordinate y.  The ghost state depends only on the grid and the
// configuration, so it is evaluated once per ghost cell on the host (compiled
// without FMA contraction, in the reference's operation order) and the device
// copies it like a flow_state_copy.
#pragma once

#include <stdexcept>
#include <vector>

namespace ibisgb {

// CubicSpline (src/util/util/cubic_spline.{h,cpp}).  The second derivatives at
// the interior knots solve the tridiagonal system of the natural spline, built
// and eliminated (Thomas algorithm) as cubic_spline.cpp:34-84 does; both end
// knots have zero second derivative.  (The reference keeps only n-2 of the n
// second derivatives and reads the last two past the end of its array; the
// values it means are the solved one at knot n-2 and zero at knot n-1.)
class NaturalSpline {
public:
    NaturalSpline() = default;
    NaturalSpline(const std::vector<double>& x, const std::vector<double>& y) : x_(x), y_(y) {
        const size_t n = x.size();
        if (n < 4) throw std::runtime_error("Insufficient points for cubic spline");
        if (y.size() != n) throw std::runtime_error("Cubic spline has different number of x and y points");
        const size_t ne = n - 2;
        std::vector<double> diag(ne, 0.0), up(ne, 0.0), rhs(ne, 0.0);
        for (size_t i = 0; i <= ne; i++) {
            const double h = x[i + 1] - x[i];
            const double s = (y[i + 1] - y[i]) / h;
            if (i < ne) {
                diag[i] += h;
                rhs[i] -= s;
            }
            if (i > 0) {
                rhs[i - 1] += s;
                diag[i - 1] += h;
                up[i - 1] += h;
            }
        }
        for (size_t i = 0; i < ne; i++) {
            rhs[i] *= 6;
            diag[i] *= 2;
        }
        for (size_t i = 1; i < ne; i++) {
            const double w = up[i - 1] / diag[i - 1];
            diag[i] = diag[i] - w * up[i - 1];
            rhs[i] = rhs[i] - w * rhs[i - 1];
        }
        m_.assign(n, 0.0);
        m_[n - 2] = rhs[ne - 1] / diag[ne - 1];
        for (size_t i = ne - 1; i-- > 0;) m_[i + 1] = (rhs[i] - up[i] * m_[i + 2]) / diag[i];
    }

    // cubic_spline.h:13-38: the end values outside [x0, x_{n-1}]
    double operator()(double t) const {
        if (t <= x_.front()) return y_.front();
        if (t >= x_.back()) return y_.back();
        size_t k = 1;
        while (x_[k] < t) k++;
        const size_t i = k - 1;
        const double dp = x_[i + 1] - t, dm = t - x_[i], h = x_[i + 1] - x_[i];
        const double a = (m_[i] * dp * dp * dp + m_[i + 1] * dm * dm * dm) / (6 * h);
        const double b = (y_[i] / h - m_[i] * h / 6) * dp;
        const double c = (y_[i + 1] / h - m_[i + 1] * h / 6) * dm;
        return a + b + c;
    }

private:
    std::vector<double> x_, y_, m_;
};

struct BoundaryLayerProfile {
    NaturalSpline vx, T;
    double p = 0.0;
};

}  // namespace ibisgb
