// Error reporting and version of the C ABI (include/qandle_gb300.h).
#include <string>

#include "qandle_gb300.h"

namespace qg {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

}  // namespace qg

extern "C" {

int qg_version(void) { return 100; }

const char* qg_last_error(void) { return qg::last_error(); }

}  // extern "C"
