// Boost.Random distributions used by the reference, over the standard
// library's (their draws differ from Boost's; the fixtures built here use no
// random draws on the compared path).  Test infrastructure.
#pragma once
#include <random>
namespace boost {
template <class T = double>
class normal_distribution {
    std::normal_distribution<T> d;

   public:
    explicit normal_distribution(T mean = 0, T sigma = 1) : d(mean, sigma) {}
    template <class E>
    T operator()(E& e) {
        return d(e);
    }
};
template <class T = double, class U = T>
class uniform_01 {
    std::uniform_real_distribution<T> d{T(0), T(1)};

   public:
    template <class E>
    T operator()(E& e) {
        return d(e);
    }
};
}  // namespace boost
