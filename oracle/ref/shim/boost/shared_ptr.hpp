// The two boost names the reference's headers use (core/common.h), mapped to the standard
// library. Test infrastructure of the oracle only.
#ifndef ORACLE_REF_BOOST_SHARED_PTR_SHIM
#define ORACLE_REF_BOOST_SHARED_PTR_SHIM
#include <memory>
namespace boost {
using std::dynamic_pointer_cast;
using std::shared_ptr;
}  // namespace boost
#endif
