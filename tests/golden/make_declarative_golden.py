"""Records tests/golden/declarative.json: for every document in
tests/golden/declarative/, the Connectome the reference's own
DeclarativeLoader + ConnectomeBuilder build from it (through
oracle/_ref/decl_dump, compiled from the reference sources by
`make -C oracle ref`), as sha256 digests of canonical arrays plus the
populations table, or the reference's error message.

    python tests/golden/make_declarative_golden.py
"""

from __future__ import annotations

import hashlib
import json
import pathlib
import subprocess
import sys
import tempfile

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
DUMP = ROOT / "oracle" / "_ref" / "decl_dump"


def canonical_from_dump(raw: bytes):
    """The dump's arrays in the canonical form canonical_arrays() gives."""
    pos = 0

    def take(dtype, count=1):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a

    n, s = (int(x) for x in take(np.uint64, 2))
    stdp = bool(take(np.uint8)[0])
    neuron_t = np.dtype([("thr", "<f4"), ("win", "<u8"), ("sim", "<f4"), ("refs", "<u8")])
    neurons = take(neuron_t, n)
    cols = {k: [] for k in ("src", "tgt", "w", "mw", "dly", "comp", "rec", "pl", "cnt")}
    codes = []
    head_t = np.dtype([("src", "<u4"), ("tgt", "<u4"), ("w", "<f4"), ("mw", "<f4"), ("dly", "<u4"),
                       ("comp", "u1"), ("rec", "u1"), ("pl", "u1"), ("cnt", "<u4")])
    for _ in range(s):
        h = take(head_t)[0]
        for k in cols:
            cols[k].append(h[k])
        codes.append(take(np.uint32, int(h["cnt"])))
    pops = {}
    for _ in range(int(take(np.uint64)[0])):
        klen = int(take(np.uint32)[0])
        key = raw[pos:pos + klen].decode()
        pos += klen
        cnt = int(take(np.uint64)[0])
        pops[key] = [int(x) for x in take(np.uint64, cnt)]
    arrays = {
        "threshold": neurons["thr"].astype(np.float32), "pattern_window_ticks": neurons["win"].astype(np.uint64),
        "similarity_threshold": neurons["sim"].astype(np.float32),
        "max_reference_patterns": neurons["refs"].astype(np.uint64),
        "source": np.array(cols["src"], np.uint32), "target": np.array(cols["tgt"], np.uint32),
        "weight": np.array(cols["w"], np.float32), "max_weight": np.array(cols["mw"], np.float32),
        "delay_ticks": np.array(cols["dly"], np.uint32), "compartment": np.array(cols["comp"], np.uint8),
        "receptor": np.array(cols["rec"], np.uint8), "plasticity_enabled": np.array(cols["pl"], np.uint8),
        "code_counts": np.array(cols["cnt"], np.uint64),
        "code_offsets": np.concatenate(codes).astype(np.uint32) if codes else np.zeros(0, np.uint32),
    }
    return n, s, stdp, arrays, pops


def canonical_arrays(c):
    """The same arrays from a snncuda_gb300 Connectome."""
    ptr = np.asarray(c.code_offset_ptr, np.uint64)
    return {
        "threshold": c.threshold, "pattern_window_ticks": c.pattern_window_ticks,
        "similarity_threshold": c.similarity_threshold, "max_reference_patterns": c.max_reference_patterns,
        "source": c.source, "target": c.target, "weight": c.weight, "max_weight": c.max_weight,
        "delay_ticks": c.delay_ticks, "compartment": c.compartment, "receptor": c.receptor,
        "plasticity_enabled": c.plasticity_enabled, "code_counts": np.diff(ptr).astype(np.uint64),
        "code_offsets": c.code_offsets,
    }


def digests(arrays):
    return {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in arrays.items()}


def record(doc: pathlib.Path):
    with tempfile.TemporaryDirectory() as tmp:
        out = pathlib.Path(tmp) / "dump.bin"
        proc = subprocess.run([str(DUMP), str(doc), str(out)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                              text=True)
        if proc.returncode == 2:
            return {"error": proc.stderr.strip()}
        if proc.returncode != 0:
            raise RuntimeError(proc.stderr)
        n, s, stdp, arrays, pops = canonical_from_dump(out.read_bytes())
    entry = {"neurons": n, "synapses": s, "stdp_enabled": stdp, "digests": digests(arrays)}
    if n <= 1000:
        entry["populations"] = {k: pops[k] for k in sorted(pops)}
    else:
        entry["populations_sizes"] = {k: len(pops[k]) for k in sorted(pops)}
    return entry


def main():
    if not DUMP.exists():
        sys.exit("oracle/_ref/decl_dump missing: run `make -C oracle ref` where the reference sources exist")
    golden = {doc.name: record(doc) for doc in sorted((HERE / "declarative").glob("*.snncuda.json"))}
    (HERE / "declarative.json").write_text(json.dumps(golden, indent=1, sort_keys=True) + "\n")
    print(f"recorded {len(golden)} documents")


if __name__ == "__main__":
    main()
