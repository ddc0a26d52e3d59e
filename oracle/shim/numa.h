/* Minimal libnuma stand-in for compiling the reference headers on a host
 * without libnuma; the checker never allocates through it. */
#pragma once
#include <stddef.h>
#include <stdlib.h>
static inline void* numa_alloc_onnode(size_t n, int node) { (void)node; return malloc(n); }
static inline void numa_free(void* p, size_t n) { (void)n; free(p); }
static inline int numa_available(void) { return -1; }
static inline void numa_tonode_memory(void*, size_t, int) {}
