// Error plumbing for the C ABI: every entry point catches, records a message
// for dp_last_error() and returns a status instead of panicking.
#pragma once

#include "setup.hpp"

#include <exception>
#include <new>
#include <string>

namespace diaphane {

void set_last_error(const std::string &message);
void clear_last_error();

template <typename F> dp_status guarded(F &&body) {
    try {
        clear_last_error();
        return body();
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return DP_ERR_OOM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return DP_ERR_INVALID;
    }
}

} // namespace diaphane
