"""Generate tests/golden/wasm_vectors.json with the reference's own Python
counter (mfah/folding.py), exactly as mfah/wasm/test_wasm.mjs:13-27 builds its
payloads: the first `count` raw prefixes at `depth`, counted to `stopDepth`.

    python tests/golden/make_wasm_vectors.py     # needs the reference checkout
"""
from __future__ import annotations

import base64
import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference checkout: $MF_REFERENCE_DIR, else `reference` beside this
# repository's checkout.
REFERENCE = Path(os.environ.get("MF_REFERENCE_DIR")
                 or Path(__file__).resolve().parents[3] / "reference")

# mfah/wasm/test_wasm.mjs:61-65
TRIPLES = [(5, 14, 20, 16), (6, 14, 20, 16), (7, 14, 28, 64)]


def main():
    # Load folding.py on its own: the mfah package __init__ pulls in Flask.
    import importlib.util

    spec = importlib.util.spec_from_file_location("ref_folding", REFERENCE / "mfah" / "folding.py")
    folding = importlib.util.module_from_spec(spec)
    sys.modules["ref_folding"] = folding
    spec.loader.exec_module(folding)
    count_payload_raw, generate_prefixes = folding.count_payload_raw, folding.generate_prefixes

    cases = []
    for n, depth, stop, count in TRIPLES:
        prefixes = generate_prefixes(n, depth)[:count]
        payload = {"n": n, "depth": depth, "stopDepth": stop, "prefixes": prefixes}
        expected = count_payload_raw(payload)
        raw = [list(base64.b64decode(p)) + [0] * (64 - depth) for p in prefixes]
        cases.append({"n": n, "depth": depth, "stopDepth": stop, "count": count,
                      "prefixes_b64": prefixes, "prefix_bytes": raw, "expected": expected})
    out = {"generated_by": "tests/golden/make_wasm_vectors.py with mfah/folding.py",
           "cases": cases}
    (HERE / "wasm_vectors.json").write_text(json.dumps(out) + "\n")
    for c in cases:
        print(c["n"], c["depth"], c["stopDepth"], c["count"], c["expected"])


if __name__ == "__main__":
    main()
