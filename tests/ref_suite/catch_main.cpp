// Catch2's runner for the reference's own test sources (the single-header
// Catch2 the reference vendors under external/catch2).
#define CATCH_CONFIG_MAIN
#include <catch.hpp>
