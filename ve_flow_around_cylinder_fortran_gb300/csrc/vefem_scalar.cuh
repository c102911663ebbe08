// Scalar type underlying a value type of the physics templates: the type
// itself for double and float, the component type for dual numbers.  The
// physics converts its double parameters to this type once, so a float
// instantiation computes in FP32 only.
#pragma once

namespace vefem {

template <class R>
struct ScalarOf {
    typedef R type;
};

}  // namespace vefem
