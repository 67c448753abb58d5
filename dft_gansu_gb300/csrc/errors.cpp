// Thread-local error message behind hf_last_error(); C++ exceptions never
// cross the C ABI (the reference throws, include/utils.hpp:91).
#include <atomic>
#include <string>

#include "internal.hpp"

namespace gb {
namespace {
thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};
}  // namespace
void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace gb

extern "C" {
const char* hf_last_error(void) { return gb::g_last_error.c_str(); }
const char* hf_version(void) { return "gansu_gb300 0.1.0 (sm_103a)"; }
long long hf_kernel_launch_count(void) { return gb::launch_count(); }
}
