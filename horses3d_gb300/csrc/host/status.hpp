// Thread-local error text behind the int status codes of the C ABI.
#pragma once
#include <string>

namespace h3d {

// Records msg as the calling thread's last error and returns code.
int fail(int code, const std::string& msg);
const char* last_error();

}  // namespace h3d
