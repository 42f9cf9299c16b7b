// flock/logger.h -- the reference's log call (src/logger.h:1-9,
// src/logger.cpp:3-6): one line "[level] => message" on stdout.
#pragma once
#include <iostream>
#include <string>

#include "structs.h"

inline void add_log_msg(std::string level, std::string log_msg) {
    std::cout << "[" << level << "] => " << log_msg << std::endl;
}
