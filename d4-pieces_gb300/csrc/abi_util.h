// abi_util.h -- error reporting shared by the extern "C" entry points: a
// failing call stores its message for d4e_last_error() (per thread) and
// returns a D4E_ERR_* code; exceptions from the engine become codes.
#pragma once

#include <new>
#include <string>

#include "../../include/d4e.h"
#include "engine.h"

namespace d4e {

int abi_fail(int code, const std::string &msg);
void abi_clear_error();

template <class F>
int abi_guarded(F &&f) {
    try {
        abi_clear_error();
        return f();
    } catch (const Error &e) {
        return abi_fail(e.code, e.what());
    } catch (const std::bad_alloc &) {
        return abi_fail(D4E_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return abi_fail(D4E_ERR_INVALID, e.what());
    }
}

}  // namespace d4e
