// Shared host-side helpers of libbh_gpu.so: status reporting.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/bh_gpu.h"

// Records `msg` as the calling thread's last error and returns `status`.
int bh_fail(int status, const std::string& msg);
// Clears the calling thread's last error.
void bh_clear_error();

// One data row of readCSV (src/io.cpp:45-70): true and the 7 values
// (mass, position, velocity) when the row parses, as std::stod parses.
bool bh_parse_csv_row(const std::string& line, double v[7]);
