"""Declarative network loading: the native `.snncuda.json` format into a
Connectome the backend consumes.

Restates, for the native JSON format, the reference's
`DeclarativeLoader::parse_only` (`src/declarative/DeclarativeLoader.cpp`)
with `parse_native_json_document` (`src/declarative/parsers/
BuiltinParsers.cpp:968-986`) and `ConnectomeBuilder::build`
(`src/declarative/Connectome.cpp:86-226`):

- the document is the top-level object, or its `snncuda` / `snnframe`
  member;
- `neuron_params`: named NeuronParamsIR sets (`threshold`,
  `pattern_window_ticks` | `window_ticks` | `window_size_ms`,
  `similarity_threshold`, `max_reference_patterns` | `max_patterns`), a
  single `default` set when absent (`BuiltinParsers.cpp:619-634`);
- `brain`: hemispheres / lobes / regions / nuclei / columns / layers /
  populations, nuclei with a `column_template` expanded over orientations x
  frequencies (`:478-614`); a `network` object with `populations` replaces it
  by one flat column (`:945-966`);
- `projections` at the document level, then inside `network` (`:658-667`,
  `:636-656`), with their defaults (pattern all_to_all, weight 1, max_weight
  2, delay 1, offsets {0}, basal, AMPA, plastic);
- `simulation`: `stdp_enabled` / `stdp.enabled` and the resident-neuron
  count (`:669-681`);
- building: neurons numbered 1.. in hierarchy order, each population
  reachable by its full path and by its short name (both keys collect the
  ids in order); a projection resolves its source and target selectors (an
  exact key, else every path ending in `/selector`, or `prefix*suffix`
  matches), then `one_to_one` pairs them up to the shorter list and every
  other pattern connects all pairs in source-major order; empty spike-code
  lists become {0}.

Numbers are converted as the reference does: `static_cast<float>` of the
double for floats, truncation toward zero for integers.

The construction is vectorized (numpy), so a projection of 1e4 x 1e4
neurons (1e8 synapses) builds in seconds.

One difference is deliberate: the reference keeps its population table in
an `std::unordered_map`, so a selector that matches several populations by
suffix or wildcard concatenates them in the hash table's iteration order,
which the C++ standard leaves unspecified.  Here such a selector
concatenates them in declaration order.  Exact names and paths, and
selectors that match one population, give the reference's Connectome
exactly (`tests/test_declarative.py` checks it against the reference's own
loader).
"""

from __future__ import annotations

import json
import math
import pathlib
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple, Union

import numpy as np

from .connectome import AMPA, APICAL, BASAL, GABA_A, GABA_B, INHIBITORY, NMDA, SOMA, Connectome


@dataclass
class NeuronParamsSpec:
    threshold: float = 1.0
    pattern_window_ticks: int = 500
    similarity_threshold: float = 0.93
    max_reference_patterns: int = 500


@dataclass
class PopulationSpec:
    name: str
    count: int
    neuron_params: str


@dataclass
class ProjectionSpec:
    name: str = "projection"
    source: str = ""
    target: str = ""
    pattern: str = "all_to_all"
    probability: float = 1.0
    weight: float = 1.0
    max_weight: float = 2.0
    delay_ticks: int = 1
    spike_code_offsets: List[int] = field(default_factory=lambda: [0])
    compartment: int = BASAL
    receptor: int = AMPA
    plasticity_enabled: bool = True
    scope: str = "global"


@dataclass
class SimulationSpec:
    timestep_ns: int = 1_000_000
    cuda_resident_neurons: int = 65536
    stdp_enabled: bool = True


@dataclass
class NetworkSpec:
    """The parsed document (the reference's NetworkIR): the population paths
    in declaration order, the projections and the parameter sets."""
    brain_name: str
    populations: List[Tuple[str, PopulationSpec]]  # (full path, population)
    hemispheres: int
    neuron_params: Dict[str, NeuronParamsSpec]
    projections: List[ProjectionSpec]
    simulation: SimulationSpec


# ---- number and field conversions (BuiltinParsers.cpp:389-428) -------------

def _is_number(v) -> bool:
    return isinstance(v, (int, float)) and not isinstance(v, bool)


def _f32(v, fallback: float) -> float:
    return float(np.float32(float(v))) if _is_number(v) else fallback


def _u64(v, fallback: int) -> int:
    if not _is_number(v) or not math.isfinite(float(v)):
        return fallback
    return int(float(v)) if float(v) >= 0 else fallback


def _str(v, fallback: str = "") -> str:
    return v if isinstance(v, str) else fallback


def _bool(v, fallback: bool) -> bool:
    return v if isinstance(v, bool) else fallback


def _u32_list(v, fallback: List[int]) -> List[int]:
    if not isinstance(v, list):
        return list(fallback)
    out = [int(float(x)) & 0xFFFFFFFF for x in v if _is_number(x)]
    return out if out else list(fallback)


def _obj(v) -> dict:
    """A JSON value seen as an object (a non-object finds nothing)."""
    return v if isinstance(v, dict) else {}


def _arr(v) -> list:
    return v if isinstance(v, list) else []


def _find_any(obj: dict, keys):
    for k in keys:
        if k in obj:
            return obj[k]
    return None


def _compartment(v, fallback: int) -> int:
    t = _str(v).lower()
    return {"soma": SOMA, "somatic": SOMA, "basal": BASAL, "apical": APICAL, "inhibitory": INHIBITORY,
            "inhibition": INHIBITORY}.get(t, fallback)


def _receptor(v, fallback: int) -> int:
    t = _str(v).lower()
    return {"ampa": AMPA, "nmda": NMDA, "gabaa": GABA_A, "gaba_a": GABA_A, "gaba-a": GABA_A, "gabab": GABA_B,
            "gaba_b": GABA_B, "gaba-b": GABA_B}.get(t, fallback)


# ---- parsing (BuiltinParsers.cpp:457-681, :945-986) --------------------------

def _neuron_params(v: dict) -> NeuronParamsSpec:
    p = NeuronParamsSpec()
    p.threshold = _f32(v.get("threshold"), p.threshold)
    p.pattern_window_ticks = _u64(_find_any(v, ("pattern_window_ticks", "window_ticks", "window_size_ms")),
                                  p.pattern_window_ticks)
    p.similarity_threshold = _f32(v.get("similarity_threshold"), p.similarity_threshold)
    p.max_reference_patterns = _u64(_find_any(v, ("max_reference_patterns", "max_patterns")),
                                    p.max_reference_patterns)
    return p


def _population(v) -> PopulationSpec:
    v = _obj(v)
    name = _str(v.get("name"), "population")
    count = _u64(v.get("count"), _u64(v.get("size"), 0))
    params = _str(v.get("neuron_params"), "default") or "default"
    return PopulationSpec(name, count, params)


def _layer(v) -> Tuple[str, List[PopulationSpec]]:
    v = _obj(v)
    return _str(v.get("name"), "Layer"), [_population(p) for p in _arr(v.get("populations"))]


def _trim_number(x: float) -> str:
    """std::to_string(double) ("%f") with trailing zeros and '.' removed."""
    text = "%f" % x
    text = text.rstrip("0")
    return text[:-1] if text.endswith(".") else text


def _columns(nucleus: dict) -> List[Tuple[str, list]]:
    cols = []
    for c in _arr(nucleus.get("columns")):
        c = _obj(c)
        cols.append((_str(c.get("name"), "Column"), [_layer(l) for l in _arr(c.get("layers"))]))
    templ = nucleus.get("column_template")
    if isinstance(templ, dict):
        orientations = [0.0]
        frequencies = [0.0]
        if isinstance(templ.get("orientations"), list):
            orientations = [float(x) for x in templ["orientations"] if _is_number(x)]
        if isinstance(templ.get("frequencies"), list):
            frequencies = [float(x) for x in templ["frequencies"] if _is_number(x)]
        pattern = _str(templ.get("naming_pattern"), "Orient_{orientation}_Freq_{frequency}")
        for o in orientations:
            for f in frequencies:
                name = pattern.replace("{orientation}", _trim_number(o), 1)
                name = name.replace("{frequency}", _trim_number(f), 1)
                cols.append((name, [_layer(l) for l in _arr(templ.get("layers"))]))
    return cols


def _brain(v, fallback_name: str):
    """(brain name, [(hemisphere, lobe, region, nucleus, column, [(layer, pops)])], hemisphere count)."""
    if not isinstance(v, dict):
        return fallback_name, [], 1
    name = _str(v.get("name"), fallback_name if fallback_name else "Brain")
    columns = []
    count = 0
    for h in map(_obj, _arr(v.get("hemispheres"))):
        count += 1
        hn = _str(h.get("name"), "Hemisphere")
        for lo in map(_obj, _arr(h.get("lobes"))):
            ln = _str(lo.get("name"), "Lobe")
            for r in map(_obj, _arr(lo.get("regions"))):
                rn = _str(r.get("name"), "Region")
                for nu in map(_obj, _arr(r.get("nuclei"))):
                    nn = _str(nu.get("name"), "Nucleus")
                    for cn, layers in _columns(nu):
                        columns.append((hn, ln, rn, nn, cn, layers))
    return name, columns, max(count, 1)


def _projection(v: dict) -> ProjectionSpec:
    p = ProjectionSpec()
    p.name = _str(v.get("name"), "projection")
    p.source = _str(v.get("source"))
    p.target = _str(v.get("target"))
    p.pattern = _str(v.get("pattern"), p.pattern)
    p.probability = _f32(v.get("probability"), p.probability)
    p.weight = _f32(v.get("weight"), p.weight)
    p.max_weight = _f32(v.get("max_weight"), p.max_weight)
    p.delay_ticks = _u64(_find_any(v, ("delay_ticks", "delay_ms", "delay")), p.delay_ticks) & 0xFFFFFFFF
    p.spike_code_offsets = _u32_list(_find_any(v, ("spike_code_offsets", "spike_pattern_offsets",
                                                   "spike_offsets")), p.spike_code_offsets)
    p.compartment = _compartment(v.get("compartment"), p.compartment)
    p.receptor = _receptor(v.get("receptor"), p.receptor)
    p.plasticity_enabled = _bool(_find_any(v, ("plasticity_enabled", "stdp_enabled")), p.plasticity_enabled)
    p.scope = _str(v.get("scope"), p.scope)
    return p


def parse_native_json(root: dict) -> NetworkSpec:
    """The parsed document of a native `.snncuda.json` (parse_native_json_document)."""
    if not isinstance(root, dict):
        raise ValueError("the document must be a JSON object")
    doc = root["snncuda"] if "snncuda" in root else root["snnframe"] if "snnframe" in root else root
    doc = _obj(doc)
    params: Dict[str, NeuronParamsSpec] = {}
    np_map = doc.get("neuron_params")
    if isinstance(np_map, dict):
        for name, v in np_map.items():
            if isinstance(v, dict):
                params[name] = _neuron_params(v)
    if not params:
        params["default"] = NeuronParamsSpec()
    brain_name, columns, hemis = _brain(doc.get("brain"), _str(doc.get("network_name"), "Brain"))
    net = doc.get("network")
    if isinstance(net, dict) and "populations" in net:
        brain_name = _str(net.get("name"), "Network")
        pops = net.get("populations")
        layer = ("Layer", [_population(p) for p in pops] if isinstance(pops, list) else [])
        columns = [("Left", "Lobe", "Region", "Nucleus", "Column", [layer])]
        hemis = 1
    populations = []
    for hn, ln, rn, nn, cn, layers in columns:
        prefix = f"{brain_name}/{hn}/{ln}/{rn}/{nn}/{cn}"
        for layer_name, pops in layers:
            for p in pops:
                populations.append((f"{prefix}/{layer_name}/{p.name}", p))
    projections = []
    for holder in (doc, net if isinstance(net, dict) else {}):
        arr = holder.get("projections")
        if isinstance(arr, list):
            projections += [_projection(p) for p in arr if isinstance(p, dict)]
    sim = SimulationSpec()
    sv = doc.get("simulation")
    if isinstance(sv, dict):
        sim.cuda_resident_neurons = _u64(_find_any(sv, ("cuda_resident_neurons", "resident_neurons")),
                                         sim.cuda_resident_neurons)
        sim.stdp_enabled = _bool(sv.get("stdp_enabled"), sim.stdp_enabled)
        if isinstance(sv.get("stdp"), dict):
            sim.stdp_enabled = _bool(sv["stdp"].get("enabled"), sim.stdp_enabled)
    return NetworkSpec(brain_name, populations, hemis, params, projections, sim)


def validate(spec: NetworkSpec) -> List[str]:
    """NetworkIR::validate (src/declarative/NetworkIR.cpp:5-33)."""
    errors = []
    if not spec.brain_name:
        errors.append("brain.name is required")
    if spec.hemispheres == 0:
        errors.append("brain must declare at least one hemisphere")
    for name, p in spec.neuron_params.items():
        if not name:
            errors.append("neuron parameter set name cannot be empty")
        if not p.threshold > 0.0:
            errors.append("neuron threshold must be positive")
    for p in spec.projections:
        if not p.name:
            errors.append("projection.name is required")
        if not p.source or not p.target:
            errors.append("projection source and target are required")
    return errors


# ---- building (Connectome.cpp:86-226) ----------------------------------------

def _ends_with_path(path: str, suffix: str) -> bool:
    return path == suffix or (len(path) > len(suffix) and path.endswith(suffix)
                              and path[len(path) - len(suffix) - 1] == "/")


def _resolve(table: Dict[str, List[np.ndarray]], selector: str) -> np.ndarray:
    if selector in table:
        return np.concatenate(table[selector]) if table[selector] else np.zeros(0, np.int64)
    parts = []
    star = selector.find("*")
    if star < 0:
        for path, ids in table.items():
            if _ends_with_path(path, selector):
                parts += ids
    else:
        prefix, suffix = selector[:star], selector[star + 1:]
        for path, ids in table.items():
            if len(path) >= len(prefix) + len(suffix) and path.startswith(prefix) and path.endswith(suffix):
                parts += ids
    return np.concatenate(parts) if parts else np.zeros(0, np.int64)


def build_connectome(spec: NetworkSpec) -> Connectome:
    """ConnectomeBuilder::build: neuron ids 1.. in hierarchy order, synapses in
    projection order.  Raises ValueError (std::invalid_argument in the
    reference) for an invalid document."""
    errors = validate(spec)
    if errors:
        raise ValueError(errors[0])
    table: Dict[str, List[np.ndarray]] = {}
    thr, win, sim, refs = [], [], [], []
    next_id = 1
    for path, pop in spec.populations:
        ids = np.arange(next_id, next_id + pop.count, dtype=np.int64)
        next_id += pop.count
        table.setdefault(path, []).append(ids)
        table.setdefault(pop.name, []).append(ids)
        p = spec.neuron_params.get(pop.neuron_params, NeuronParamsSpec())
        thr.append(np.full(pop.count, p.threshold, np.float32))
        win.append(np.full(pop.count, p.pattern_window_ticks, np.uint64))
        sim.append(np.full(pop.count, p.similarity_threshold, np.float32))
        refs.append(np.full(pop.count, p.max_reference_patterns, np.uint64))
    cat = lambda xs, dt: np.concatenate(xs).astype(dt, copy=False) if xs else np.zeros(0, dt)  # noqa: E731
    src_l, tgt_l, w_l, mw_l, d_l, c_l, r_l, pl_l, k_l, codes_l = [], [], [], [], [], [], [], [], [], []
    for proj in spec.projections:
        s = _resolve(table, proj.source)
        t = _resolve(table, proj.target)
        if s.size == 0 or t.size == 0:
            continue
        if proj.pattern == "one_to_one":
            m = min(s.size, t.size)
            src, tgt = s[:m], t[:m]
        else:
            src = np.repeat(s, t.size)
            tgt = np.tile(t, s.size)
        n = src.size
        offs = proj.spike_code_offsets if proj.spike_code_offsets else [0]
        src_l.append(src - 1)
        tgt_l.append(tgt - 1)
        w_l.append(np.full(n, proj.weight, np.float32))
        mw_l.append(np.full(n, proj.max_weight, np.float32))
        d_l.append(np.full(n, proj.delay_ticks, np.uint32))
        c_l.append(np.full(n, proj.compartment, np.uint8))
        r_l.append(np.full(n, proj.receptor, np.uint8))
        pl_l.append(np.full(n, 1 if proj.plasticity_enabled else 0, np.uint8))
        k_l.append(np.full(n, len(offs), np.uint64))
        codes_l.append(np.tile(np.asarray(offs, np.uint32), n))
    counts = cat(k_l, np.uint64)
    ptr = np.zeros(counts.size + 1, np.uint64)
    np.cumsum(counts, out=ptr[1:])
    populations = {k: [int(x) for x in np.concatenate(v)] for k, v in table.items()}
    return Connectome(
        threshold=cat(thr, np.float32), pattern_window_ticks=cat(win, np.uint64),
        similarity_threshold=cat(sim, np.float32), max_reference_patterns=cat(refs, np.uint64),
        source=cat(src_l, np.uint32), target=cat(tgt_l, np.uint32), weight=cat(w_l, np.float32),
        max_weight=cat(mw_l, np.float32), delay_ticks=cat(d_l, np.uint32), compartment=cat(c_l, np.uint8),
        receptor=cat(r_l, np.uint8), plasticity_enabled=cat(pl_l, np.uint8), code_offset_ptr=ptr,
        code_offsets=cat(codes_l, np.uint32), populations=populations)


def load(path_or_document: Union[str, pathlib.Path, dict]) -> Tuple[Connectome, SimulationSpec]:
    """DeclarativeLoader::parse_only + ConnectomeBuilder::build for a native
    `.snncuda.json` file (or an already parsed document): the Connectome and
    the simulation settings (`stdp_enabled` maps to snncuda_config.stdp_enabled)."""
    if isinstance(path_or_document, dict):
        root = path_or_document
    else:
        # a repeated key keeps its first value, as the reference's parser
        # (object.emplace) does
        root = json.loads(pathlib.Path(path_or_document).read_text(),
                          object_pairs_hook=lambda pairs: {k: v for k, v in reversed(pairs)})
    spec = parse_native_json(root)
    return build_connectome(spec), spec.simulation
