// Typed host-side errors.  They never cross the C ABI: every exported entry point catches
// them, stores the message for spn_last_error() and returns a negative status code.
// The categories mirror the reference's Exception::Type (src/lib/Exception.hpp:17-121).
#pragma once
#include <stdexcept>
#include <string>

namespace spn {

enum class ErrorType : int {
    Argument = -2,        // invalid argument / descriptor
    Initialization = -3,  // malformed task, lattice or model definition
    IO = -4,              // file cannot be opened, read or written
    Cuda = -5,            // CUDA runtime failure (allocation, launch, copy)
    Device = -6,          // device-side status word reported a problem
    Internal = -7,        // consistency check failed
    Unsupported = -8,     // size or feature beyond what the library supports
};

class Error : public std::runtime_error {
public:
    Error(ErrorType t, const std::string &msg) : std::runtime_error(msg), type(t) {}
    ErrorType type;
};

}  // namespace spn
