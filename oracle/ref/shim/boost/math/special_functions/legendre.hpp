// Legendre polynomials P_l(x) and their derivatives, with the names and call
// shapes of Boost.Math's legendre_p / legendre_p_prime, written for this
// project so that the reference compiles where Boost is not installed.
//
// TEST INFRASTRUCTURE ONLY (backs the CPU reference build).
//
// Method (Bonnet's three-term recurrence, any numerical-analysis text):
//   P_0 = 1, P_1 = x, (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1};
// the derivative from the recurrence differentiated term by term:
//   P'_0 = 0, P'_1 = 1, P'_{k+1} = P'_{k-1} + (2k+1) P_k.
// Negative degrees use P_{-l-1} = P_l.
#ifndef SEM_REF_BOOST_LEGENDRE_SHIM
#define SEM_REF_BOOST_LEGENDRE_SHIM

namespace boost
{
namespace math
{

template <typename T>
T legendre_p(int l, T x)
{
    if (l < 0) l = -l - 1;
    if (l == 0) return T(1);
    T p0 = T(1), p1 = x;
    for (int k = 1; k < l; ++k)
    {
        T p2 = (T(2 * k + 1) * x * p1 - T(k) * p0) / T(k + 1);
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

template <typename T>
T legendre_p_prime(int l, T x)
{
    if (l < 0) l = -l - 1;
    if (l == 0) return T(0);
    T p0 = T(1), p1 = x;      // P_{k-1}, P_k
    T d0 = T(0), d1 = T(1);   // P'_{k-1}, P'_k
    for (int k = 1; k < l; ++k)
    {
        T p2 = (T(2 * k + 1) * x * p1 - T(k) * p0) / T(k + 1);
        T d2 = d0 + T(2 * k + 1) * p1;
        p0 = p1;
        p1 = p2;
        d0 = d1;
        d1 = d2;
    }
    return d1;
}

}  // namespace math
}  // namespace boost

#endif
