// Exception guards of the C ABI (pc_api.cpp, pc_io.cpp).
#pragma once

#include <exception>
#include <new>
#include <string>

// C++ exceptions never cross the C ABI: every exported function that returns a status
// wraps its body in PC_GUARD_BEGIN / PC_GUARD_END(ctx) (or PC_GUARD_END_NOCTX); a host
// allocation failure becomes PC_ERR_NOMEM and any other exception PC_ERR_INTERNAL.
#define PC_GUARD_BEGIN try {
#define PC_GUARD_END(ctx)                                                                   \
  }                                                                                         \
  catch (const std::bad_alloc&) {                                                           \
    return fail(ctx, PC_ERR_NOMEM, "host allocation failed");                               \
  }                                                                                         \
  catch (const std::exception& e) {                                                         \
    return fail(ctx, PC_ERR_INTERNAL, std::string("internal: ") + e.what());                \
  }                                                                                         \
  catch (...) {                                                                             \
    return fail(ctx, PC_ERR_INTERNAL, "internal: unknown exception");                       \
  }
#define PC_GUARD_END_NOCTX                                                                  \
  }                                                                                         \
  catch (const std::bad_alloc&) {                                                           \
    return PC_ERR_NOMEM;                                                                    \
  }                                                                                         \
  catch (...) {                                                                             \
    return PC_ERR_INTERNAL;                                                                 \
  }
