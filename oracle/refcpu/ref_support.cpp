/*
 * The particle tables the reference declares in hardCoded.cuh:15-19 but whose
 * data file (hardCoded.cu) is not part of the reference tree.  The tables are
 * filled from the oracle's particle stream (pump_oracle.c) with seed
 * PUMPREF_SEED (default 0x9E3779B97F4A7C15) and PUMPREF_TABLE_ROWS rows
 * (default 400; the reference's arrays hold the first 100).
 *
 * Test infrastructure only.
 */
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "../pump_oracle.h"

float xcomb[2048 * 100 * 3];
float xcombTime[100 * 2048 * 3];

namespace {
std::vector<float> g_ext;
int g_rows = 100;

struct Init {
  Init() {
    const char *s = std::getenv("PUMPREF_SEED");
    uint64_t seed = s ? std::strtoull(s, nullptr, 0) : 0x9E3779B97F4A7C15ull;
    const char *r = std::getenv("PUMPREF_TABLE_ROWS");
    g_rows = r ? std::atoi(r) : 400;
    if (g_rows < 100) g_rows = 100;
    g_ext.resize((size_t)g_rows * 2048 * 3);
    orc_particle_tables(seed, 2048, g_rows, g_ext.data(), nullptr);
    std::vector<float> pm((size_t)2048 * 100 * 3);
    orc_particle_tables(seed, 2048, 100, nullptr, pm.data());
    for (size_t i = 0; i < pm.size(); ++i) xcomb[i] = pm[i];
    for (size_t i = 0; i < (size_t)100 * 2048 * 3; ++i) xcombTime[i] = g_ext[i];
  }
} g_init;
}  // namespace

extern "C" const float *refsupport_table_tmajor(int *rows, int *particles) {
  *rows = g_rows;
  *particles = 2048;
  return g_ext.data();
}

