"""Connectome input for the GB300 backend.

`Connectome` is the flattened network the engine consumes: per-neuron
parameters and per-synapse arrays in Connectome vector order, the layout of
the reference's declarative::Connectome (declarative/Connectome.h:13-37),
stored as numpy structure-of-arrays.  Neuron and synapse ids follow the
reference: dense 1-based ids (ConnectomeBuilder, Connectome.cpp:137-139);
array index = id - 1.

`NetworkBuilder` restates the reference ConnectomeBuilder::build
(Connectome.cpp:131-229) for a flat list of populations: neurons are numbered
in population declaration order, each projection expands `one_to_one` or
`all_to_all` over its resolved populations, then explicit connections follow;
synapse ids are assigned in that order.  Population selectors are the
population names (the reference additionally indexes hierarchy paths, which
only name things and never change ids or order).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

SOMA, BASAL, APICAL, INHIBITORY = 0, 1, 2, 3      # snn::DendriticCompartment
AMPA, NMDA, GABA_A, GABA_B = 0, 1, 2, 3           # snn::ReceptorType


@dataclass
class NeuronParams:
    """declarative::NeuronParamsIR (NetworkIR.h:14-19) defaults."""
    threshold: float = 1.0
    pattern_window_ticks: int = 500
    similarity_threshold: float = 0.93
    max_reference_patterns: int = 500


@dataclass
class Connectome:
    threshold: np.ndarray                 # float32 [N]
    pattern_window_ticks: np.ndarray      # uint64 [N]
    similarity_threshold: np.ndarray      # float32 [N]
    max_reference_patterns: np.ndarray    # uint64 [N]
    source: np.ndarray                    # uint32 [S], 0-based neuron index
    target: np.ndarray                    # uint32 [S]
    weight: np.ndarray                    # float32 [S]
    max_weight: np.ndarray                # float32 [S]
    delay_ticks: np.ndarray               # uint32 [S]
    compartment: np.ndarray               # uint8 [S]
    receptor: np.ndarray                  # uint8 [S]
    plasticity_enabled: np.ndarray        # uint8 [S]
    code_offset_ptr: Optional[np.ndarray] = None   # uint64 [S+1]; None = all {0}
    code_offsets: Optional[np.ndarray] = None      # uint32
    populations: Dict[str, List[int]] = field(default_factory=dict)  # name -> 1-based ids

    @property
    def neuron_count(self) -> int:
        return int(self.threshold.shape[0])

    @property
    def synapse_count(self) -> int:
        return int(self.source.shape[0])

    def validate(self) -> None:
        n, s = self.neuron_count, self.synapse_count
        for name in ("pattern_window_ticks", "similarity_threshold", "max_reference_patterns"):
            if getattr(self, name).shape != (n,):
                raise ValueError(f"{name} must have shape ({n},)")
        for name in ("target", "weight", "max_weight", "delay_ticks", "compartment", "receptor",
                     "plasticity_enabled"):
            if getattr(self, name).shape != (s,):
                raise ValueError(f"{name} must have shape ({s},)")
        if (self.code_offset_ptr is None) != (self.code_offsets is None):
            raise ValueError("code_offset_ptr and code_offsets go together")
        if self.code_offset_ptr is not None and self.code_offset_ptr.shape != (s + 1,):
            raise ValueError(f"code_offset_ptr must have shape ({s + 1},)")

    def spike_codes(self, synapse_index: int) -> List[int]:
        """Spike-code offsets of one synapse ({0} when empty, as the reference)."""
        if self.code_offset_ptr is None:
            return [0]
        b, e = int(self.code_offset_ptr[synapse_index]), int(self.code_offset_ptr[synapse_index + 1])
        return [int(v) for v in self.code_offsets[b:e]] if e > b else [0]

    def copy_arrays(self) -> "Connectome":
        return Connectome(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                             for k, v in self.__dict__.items()})


@dataclass
class Projection:
    """declarative::ProjectionIR (NetworkIR.h:62-76)."""
    source: str
    target: str
    pattern: str = "all_to_all"
    weight: float = 1.0
    max_weight: float = 2.0
    delay_ticks: int = 1
    spike_code_offsets: Sequence[int] = (0,)
    compartment: int = BASAL
    receptor: int = AMPA
    plasticity_enabled: bool = True
    name: str = ""


@dataclass
class ExplicitConnection:
    """declarative::ExplicitConnectionIR (NetworkIR.h:78-90)."""
    source_population: str
    source_index: int
    target_population: str
    target_index: int
    weight: float = 1.0
    max_weight: float = 2.0
    delay_ticks: int = 1
    spike_code_offsets: Sequence[int] = (0,)
    compartment: int = BASAL
    receptor: int = AMPA
    plasticity_enabled: bool = True


class NetworkBuilder:
    """Flat-population restatement of ConnectomeBuilder::build."""

    def __init__(self) -> None:
        self.neuron_params: Dict[str, NeuronParams] = {}
        self._populations: List[tuple] = []
        self.projections: List[Projection] = []
        self.explicit_connections: List[ExplicitConnection] = []

    def add_population(self, name: str, count: int, neuron_params: str = "default") -> "NetworkBuilder":
        self._populations.append((name, int(count), neuron_params))
        return self

    def build(self) -> Connectome:
        populations: Dict[str, List[int]] = {}
        thr, win, sim, refs = [], [], [], []
        next_id = 1
        for name, count, params_name in self._populations:
            params = self.neuron_params.get(params_name, NeuronParams())
            ids = populations.setdefault(name, [])
            for _ in range(count):
                ids.append(next_id)
                next_id += 1
                thr.append(params.threshold)
                win.append(params.pattern_window_ticks)
                sim.append(params.similarity_threshold)
                refs.append(params.max_reference_patterns)

        syn: List[tuple] = []

        def add(src: int, tgt: int, spec) -> None:
            codes = list(spec.spike_code_offsets) or [0]
            syn.append((src - 1, tgt - 1, spec.weight, spec.max_weight, spec.delay_ticks,
                        spec.compartment, spec.receptor, 1 if spec.plasticity_enabled else 0, codes))

        for p in self.projections:
            sources, targets = populations.get(p.source, []), populations.get(p.target, [])
            if not sources or not targets:
                continue
            if p.pattern == "one_to_one":
                for i in range(min(len(sources), len(targets))):
                    add(sources[i], targets[i], p)
            else:
                for s in sources:
                    for t in targets:
                        add(s, t, p)
        for c in self.explicit_connections:
            sp, tp = populations.get(c.source_population, []), populations.get(c.target_population, [])
            if c.source_index >= len(sp) or c.target_index >= len(tp):
                continue
            add(sp[c.source_index], tp[c.target_index], c)

        ptr = np.zeros(len(syn) + 1, dtype=np.uint64)
        flat: List[int] = []
        for i, s in enumerate(syn):
            flat.extend(s[8])
            ptr[i + 1] = len(flat)

        def col(k, dtype):
            return np.array([s[k] for s in syn], dtype=dtype)

        return Connectome(
            threshold=np.array(thr, dtype=np.float32),
            pattern_window_ticks=np.array(win, dtype=np.uint64),
            similarity_threshold=np.array(sim, dtype=np.float32),
            max_reference_patterns=np.array(refs, dtype=np.uint64),
            source=col(0, np.uint32), target=col(1, np.uint32),
            weight=col(2, np.float32), max_weight=col(3, np.float32),
            delay_ticks=col(4, np.uint32), compartment=col(5, np.uint8),
            receptor=col(6, np.uint8), plasticity_enabled=col(7, np.uint8),
            code_offset_ptr=ptr, code_offsets=np.array(flat, dtype=np.uint32),
            populations=populations,
        )
