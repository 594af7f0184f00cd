// Batched assembly of many GEPs in one persistent launch (assemble_batch.cu).
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "device.h"

namespace fem2d {

struct LaunchShape {
  int threads;       // threads per CTA
  int ctas_per_sm;   // grid = ctas_per_sm x SMs (capped by the work)
};

struct BatchMember {
  const HostGEP* h;
  DeviceGEP* d;   // uploaded (device_upload); A and B are written in place
};

struct BatchReport {
  float ms_tables = 0, ms_values = 0;
  LaunchShape shape{0, 0};
  int64_t total_entries = 0, total_codes = 0;
  std::string key;
};

// Tables of every member in one launch, then the values of every member in one persistent launch.
// With autotune set, the launch shape is looked up in (or timed into) the per-process cache.
void batch_assemble(Ctx& c, const std::vector<BatchMember>& members, bool autotune, BatchReport* rep);

std::string tune_export();                 // "key threads ctas_per_sm" lines
int tune_import(const std::string& text);  // returns the number of entries read
void tune_clear();

}  // namespace fem2d
