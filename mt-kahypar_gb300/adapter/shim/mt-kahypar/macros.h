// Minimal stand-in for Mt-KaHyPar's mt-kahypar/macros.h (debug assertions off).
#pragma once
#define ASSERT(...)
