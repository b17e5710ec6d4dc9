// abi_guard.h -- keeps C++ exceptions from crossing the C ABI.
//
// Every extern "C" entry point returns an int status.  Host code behind it uses the
// standard library (vectors, strings, mutexes), which can throw std::bad_alloc or
// std::system_error; an exception that left an extern "C" function would end the
// caller's process through std::terminate.  RG_GUARD(expr) evaluates expr and returns
// its status, turning a bad_alloc into RG_ERR_NOMEM and anything else into RG_ERR_STATE,
// with the message available from rg_last_error().
#pragma once

#include <new>
#include <string>

namespace redgb {
int set_error(int code, const std::string& msg);
}

#define RG_GUARD(expr)                                                                    \
    try {                                                                                 \
        return (expr);                                                                    \
    } catch (const std::bad_alloc&) {                                                     \
        return ::redgb::set_error(RG_ERR_NOMEM, "host allocation failed");                \
    } catch (...) {                                                                       \
        return ::redgb::set_error(RG_ERR_STATE, "unexpected exception");                  \
    }
