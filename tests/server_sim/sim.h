// Host-only stand-in engine for driving the query server without a GPU
// (test infrastructure; see mock_engine.cpp).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include "ascetic.h"

uint32_t sim_value(asc_algo algo, uint32_t source, uint64_t v);
void sim_reset(uint64_t budget, uint32_t fail_source);
uint64_t sim_violations(char *first, size_t n);
uint64_t sim_bytes();
asc_graph *sim_graph(uint64_t V);
void sim_graph_free(asc_graph *g);
