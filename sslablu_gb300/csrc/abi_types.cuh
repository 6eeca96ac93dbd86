// Opaque handle types of the C ABI and the exception-to-status guard shared
// by the translation units that define extern "C" entry points.
#pragma once
#include <new>
#include <string>

#include "../../include/slablu.h"
#include "tridiag.cuh"

struct slu_handle_s {
  slu::Handle h;
};
struct slu_hbs_s {
  slu::Hbs H;
};
struct slu_solve_plan_s {
  slu::SolvePlan P;
};
struct slu_refine_plan_s {
  std::unique_ptr<slu::GroupRefinePlan> P;
};
struct slu_dense_rb_s {
  slu::RbSolver S;
  bool thomas = false;
};

namespace slu {

// Message of the most recent failure on the calling thread (slu_last_error).
std::string& thread_error();

// Runs f, turning exceptions into status codes; no exception crosses the ABI.
template <class F>
int guard_call(slu_handle_t h, F&& f) {
  try {
    f();
    return SLU_OK;
  } catch (const Error& e) {
    thread_error() = e.what();
    if (h) h->h.last_error = thread_error();
    return e.code;
  } catch (const std::bad_alloc&) {
    thread_error() = "host allocation failed";
    return SLU_ERR_ALLOC;
  } catch (const std::exception& e) {
    thread_error() = e.what();
    return SLU_ERR_ARG;
  } catch (...) {
    thread_error() = "unknown error";
    return SLU_ERR_ARG;
  }
}

}  // namespace slu
