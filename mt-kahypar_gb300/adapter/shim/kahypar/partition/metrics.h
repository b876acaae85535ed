// Minimal stand-in for KaHyPar's kahypar::Metrics bookkeeping as Mt-KaHyPar's
// refiners use it (getMetric / updateMetric for the km1 and cut objectives,
// and the imbalance field).
#pragma once

#include <cstdint>

namespace kahypar {

enum class Mode : uint8_t { recursive_bisection, direct_kway, UNDEFINED };
enum class Objective : uint8_t { cut, km1, UNDEFINED };

struct Metrics {
  int32_t cut = 0;
  int32_t km1 = 0;
  double imbalance = 0.0;

  int32_t getMetric(Mode, Objective objective) const { return objective == Objective::cut ? cut : km1; }
  void updateMetric(int32_t value, Mode, Objective objective) {
    if (objective == Objective::cut)
      cut = value;
    else
      km1 = value;
  }
};

}  // namespace kahypar
