// Shared host-side helpers of libbh_gpu.so: status reporting.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/bh_gpu.h"

// Records `msg` as the calling thread's last error and returns `status`.
int bh_fail(int status, const std::string& msg);
// Clears the calling thread's last error.
void bh_clear_error();
