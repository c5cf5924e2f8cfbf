// Links SNNCuda::snncuda, prints the version and CUDA availability through
// the reference's include path, then runs the reference's three-neuron
// propagation chain (propagation_tests.cpp: fires at ticks 0, 2 and 5)
// through the C ABI when a device is available.
#include <cstdint>
#include <iostream>

#include "snncuda/core/Version.h"
#include "snncuda_gb300.h"

int main() {
    std::cout << "version=" << snncuda::core::version() << " cuda_available=" << snncuda::core::cuda_available()
              << " has_cuda_define=" << SNNCUDA_HAS_CUDA << '\n';
    const float threshold[3] = {1.0F, 1.0F, 1.0F};
    const uint64_t window[3] = {500, 500, 500};
    const float similarity[3] = {0.93F, 0.93F, 0.93F};
    const uint64_t refs[3] = {500, 500, 500};
    const uint32_t source[2] = {0, 1}, target[2] = {1, 2}, delay[2] = {2, 3};
    const float weight[2] = {1.0F, 1.0F}, max_weight[2] = {2.0F, 2.0F};
    const uint8_t comp[2] = {SNNCUDA_COMPARTMENT_SOMA, SNNCUDA_COMPARTMENT_SOMA};
    const uint8_t rec[2] = {SNNCUDA_RECEPTOR_AMPA, SNNCUDA_RECEPTOR_AMPA};
    const uint8_t plastic[2] = {0, 0};
    const snncuda_network net{3,      threshold, window, similarity, refs, 2,       source, target,
                              weight, max_weight, delay, comp,       rec,  plastic, nullptr, nullptr};
    snncuda_config cfg;
    snncuda_config_default(&cfg);
    cfg.raster_capacity = 16;
    snncuda_sim* sim = nullptr;
    const int rc = snncuda_sim_create(&net, &cfg, &sim);
    std::cout << "create=" << rc << '\n';
    if (rc != SNNCUDA_OK) return 0;
    const uint32_t n0 = 0;
    const uint64_t t0 = 0;
    const float w0 = 1.0F;
    int status = snncuda_sim_inject(sim, 1, &n0, &t0, &w0);
    if (status == SNNCUDA_OK) status = snncuda_sim_run_until(sim, 10);
    snncuda_counters c{};
    if (status == SNNCUDA_OK) status = snncuda_sim_counters(sim, &c);
    uint64_t ticks[3] = {0, 0, 0};
    uint32_t neurons[3] = {0, 0, 0};
    if (status == SNNCUDA_OK) status = snncuda_sim_read_raster(sim, 0, 3, ticks, neurons);
    std::cout << "status=" << status << " delivered=" << c.delivered_spikes << " fired=" << c.fired_spikes
              << " fires=" << ticks[0] << ':' << neurons[0] << ',' << ticks[1] << ':' << neurons[1] << ','
              << ticks[2] << ':' << neurons[2] << '\n';
    snncuda_sim_destroy(sim);
    return 0;
}
