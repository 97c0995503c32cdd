// TEST INFRASTRUCTURE ONLY.  Stands in for the header the reference's CMake
// build generates from src/cmake_config.h.in, with the cache defaults of
// src/CMakeLists.txt:32-35.
#pragma once
#define SPRAY_RAY_DOMAIN_LIST_SIZE 16
#define SPRAY_SPECU_HISTORY_SIZE 4
#define SPRAY_SHADOW_TRANSPARENCY 0.3f
#define SPRAY_L1_CACHE_LINE_SIZE 64
