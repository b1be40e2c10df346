// boost::shared_ptr as std::shared_ptr (test infrastructure for building the reference)
#pragma once
#include <memory>
namespace boost {
using std::dynamic_pointer_cast;
using std::shared_ptr;
using std::static_pointer_cast;
}
