// boost::mt19937 as std::mt19937 (same generator; test infrastructure).
#pragma once
#include <random>
namespace boost {
typedef std::mt19937 mt19937;
}
