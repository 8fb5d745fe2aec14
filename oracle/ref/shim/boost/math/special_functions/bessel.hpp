// Modified Bessel function of the first kind I_nu(x) for integer order, with
// the name of Boost.Math's cyl_bessel_i; only the reference's unit test of
// the quadrature rule uses it (I_0(1)).
//
// TEST INFRASTRUCTURE ONLY (backs the CPU reference build).
//
// Method: the power series I_n(x) = sum_k (x/2)^(2k+n) / (k! (k+n)!),
// summed until the terms no longer change the sum.
#ifndef SEM_REF_BOOST_BESSEL_SHIM
#define SEM_REF_BOOST_BESSEL_SHIM

#include <cmath>

namespace boost
{
namespace math
{

template <typename T1, typename T2>
double cyl_bessel_i(T1 nu, T2 x)
{
    const int n = static_cast<int>(nu);
    const double h = 0.5 * static_cast<double>(x);
    double term = 1.0;
    for (int k = 1; k <= n; ++k) term *= h / k;
    double sum = term;
    for (int k = 1; k < 500; ++k)
    {
        term *= h * h / (double(k) * double(k + n));
        const double next = sum + term;
        if (next == sum) break;
        sum = next;
    }
    return sum;
}

}  // namespace math
}  // namespace boost

#endif
