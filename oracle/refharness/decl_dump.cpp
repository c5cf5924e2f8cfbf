// ORACLE -- test infrastructure only.  Loads a declarative network file with
// the reference's own DeclarativeLoader::parse_only and
// ConnectomeBuilder::build (compiled unmodified from the reference sources)
// and writes the resulting Connectome in a flat binary form that
// tests/golden/make_declarative_golden.py turns into fixtures:
//   u64 neuron_count, u64 synapse_count, u8 stdp_enabled,
//   per neuron:  f32 threshold, u64 window, f32 similarity, u64 max_refs
//   per synapse: u32 source-1, u32 target-1, f32 weight, f32 max_weight,
//                u32 delay, u8 compartment, u8 receptor, u8 plastic,
//                u32 code count, u32 codes...
//   populations: u64 count, then per population: u32 key length, key bytes,
//                u64 id count, u64 ids...
//   decl_dump <network file> <output file>; exit status 2 and the message on
//   stderr when the reference rejects the document.
#include <cstdint>
#include <cstdio>
#include <exception>
#include <fstream>
#include <iostream>

#include "snncuda/declarative/Connectome.h"
#include "snncuda/declarative/DeclarativeLoader.h"

namespace {

template <typename T>
void put(std::ofstream& out, T v) {
    out.write(reinterpret_cast<const char*>(&v), sizeof(v));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::cerr << "usage: decl_dump <network file> <output file>\n";
        return 1;
    }
    using namespace snncuda::declarative;
    try {
        const DeclarativeLoader loader;
        const NetworkIR ir = loader.parse_only(argv[1]);
        const Connectome c = ConnectomeBuilder{}.build(ir);
        std::ofstream out(argv[2], std::ios::binary);
        put<uint64_t>(out, c.neurons.size());
        put<uint64_t>(out, c.synapses.size());
        put<uint8_t>(out, ir.simulation.stdp_enabled ? 1 : 0);
        for (const auto& n : c.neurons) {
            put<float>(out, n.params.threshold);
            put<uint64_t>(out, n.params.pattern_window_ticks);
            put<float>(out, n.params.similarity_threshold);
            put<uint64_t>(out, n.params.max_reference_patterns);
        }
        for (const auto& s : c.synapses) {
            put<uint32_t>(out, static_cast<uint32_t>(s.source - 1));
            put<uint32_t>(out, static_cast<uint32_t>(s.target - 1));
            put<float>(out, s.weight);
            put<float>(out, s.max_weight);
            put<uint32_t>(out, s.delay_ticks);
            put<uint8_t>(out, static_cast<uint8_t>(s.compartment));
            put<uint8_t>(out, static_cast<uint8_t>(s.receptor));
            put<uint8_t>(out, s.plasticity_enabled ? 1 : 0);
            put<uint32_t>(out, static_cast<uint32_t>(s.spike_code_offsets.size()));
            for (uint32_t v : s.spike_code_offsets) put<uint32_t>(out, v);
        }
        put<uint64_t>(out, c.populations.size());
        for (const auto& [key, ids] : c.populations) {
            put<uint32_t>(out, static_cast<uint32_t>(key.size()));
            out.write(key.data(), static_cast<std::streamsize>(key.size()));
            put<uint64_t>(out, ids.size());
            for (auto id : ids) put<uint64_t>(out, id);
        }
    } catch (const std::exception& ex) {
        std::cerr << ex.what() << "\n";
        return 2;
    }
    return 0;
}
