// boost::variate_generator (test infrastructure)
#pragma once
#include <boost/random/normal_distribution.hpp>
namespace boost {
template <class Engine, class Dist>
class variate_generator {
    Engine e;
    Dist d;

   public:
    variate_generator(Engine eng, Dist dist) : e(eng), d(dist) {}
    double operator()() { return d(e); }
};
}  // namespace boost
