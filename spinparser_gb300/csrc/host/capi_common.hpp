// Exception-to-status translation shared by every exported entry point.
#pragma once
#include <exception>
#include <new>
#include <string>
#include "error.hpp"

namespace spn {

void set_last_error(const std::string &msg);

// Runs `body`; maps spn::Error to its status code, anything else to SPN_E_INTERNAL.
template <class F>
int guarded(F &&body) {
    try {
        body();
        return 0;
    } catch (const Error &e) {
        set_last_error(e.what());
        return int(e.type);
    } catch (const std::bad_alloc &) {
        set_last_error("host out of memory");
        return int(ErrorType::Internal);
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return int(ErrorType::Internal);
    } catch (...) {
        set_last_error("unknown error");
        return int(ErrorType::Internal);
    }
}

}  // namespace spn
