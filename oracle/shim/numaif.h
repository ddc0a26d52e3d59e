/* Minimal numaif.h stand-in (mbind is never called by the checker). */
#pragma once
static inline long mbind(void*, unsigned long, int, const unsigned long*, unsigned long, unsigned) { return 0; }
#define MPOL_BIND 2
#define MPOL_MF_STRICT 1
#define MPOL_MF_MOVE 2
