"""Generate tests/golden/jsonl_summaries.json: the reference's own
`summarize_jsonl` and `parse_result` (modal_sym.py:28-77) run on a set of
synthetic sweep files and stdout texts.

    python tests/golden/make_jsonl_summaries.py

modal_sym.py imports the `modal` cloud SDK at the top, which is not
installed here, so the two functions are taken out of the file by name with
`ast` and run on their own (they only need json and pathlib).  The sweep
files are written into the fixture next to the reference's answers, so the
test needs nothing but this JSON file.
"""
from __future__ import annotations

import ast
import json
import os
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference checkout: $MF_REFERENCE_DIR, else `reference` beside this
# repository's checkout.
REFERENCE = Path(os.environ.get("MF_REFERENCE_DIR")
                 or Path(__file__).resolve().parents[3] / "reference")


def reference_functions():
    src = (REFERENCE / "modal_sym.py").read_text()
    tree = ast.parse(src)
    keep = [node for node in tree.body
            if isinstance(node, ast.FunctionDef) and node.name in ("parse_result", "summarize_jsonl")]
    module = ast.Module(body=keep, type_ignores=[])
    env = {"json": json, "Path": Path}
    exec(compile(module, str(REFERENCE / "modal_sym.py"), "exec"), env)
    return env["parse_result"], env["summarize_jsonl"]


def row(start, size, count):
    return json.dumps({"completed_hint": size, "count": str(count), "expanded_n": 36,
                       "max_cases": size, "n": 8, "start_case": start,
                       "stderr_tail": "", "threads": 16, "wall_s": 1.0}, sort_keys=True)


def cases():
    """(name, jsonl text or None for a missing file, total_cases, chunk_size)."""
    out = []
    out.append(("complete", "\n".join(row(s, 10, s + 1) for s in range(0, 50, 10)) + "\n", 50, 10))
    out.append(("ragged_last_chunk", "\n".join(row(s, 10, 7 * s) for s in range(0, 45, 10)) + "\n",
                45, 10))
    out.append(("duplicates_and_blank_lines",
                "\n".join([row(0, 10, 1), "", row(10, 10, 2), row(10, 10, 3), "   ",
                           row(20, 10, 4)]) + "\n", 30, 10))
    out.append(("missing_and_extra", "\n".join([row(0, 10, 5), row(25, 10, 6)]) + "\n", 30, 10))
    out.append(("many_missing", row(0, 1, 9) + "\n", 100, 1))
    out.append(("many_duplicates", "\n".join(row(0, 5, k) for k in range(30)) + "\n", 5, 5))
    out.append(("big_counts", "\n".join(row(s, 100, 10**30 + s) for s in range(0, 300, 100)) + "\n",
                300, 100))
    out.append(("empty_file", "", 20, 10))
    out.append(("no_file", None, 20, 10))
    return out


STDOUTS = ["152870282240\n", "noise\n  152870282240 \n99\n", "Total: 12\n", "", "\n\n7\n",
           "-5\n12\n", "1 2\n3\n"]


def main():
    parse_result, summarize_jsonl = reference_functions()
    fixture = {"generated_by": "tests/golden/make_jsonl_summaries.py (modal_sym.py:28-77)",
               "summaries": [], "parse_result": []}
    with tempfile.TemporaryDirectory() as tmp:
        for name, text, total, size in cases():
            path = Path(tmp) / f"{name}.jsonl"
            if text is not None:
                path.write_text(text, encoding="utf-8")
            got = summarize_jsonl(path, total, size)
            got["path"] = f"{name}.jsonl"
            fixture["summaries"].append({"name": name, "jsonl": text, "total_cases": total,
                                         "chunk_size": size, "summary": got})
    for text in STDOUTS:
        fixture["parse_result"].append({"stdout": text, "result": parse_result(text)})
    (HERE / "jsonl_summaries.json").write_text(json.dumps(fixture, indent=1) + "\n")
    print(f"{len(fixture['summaries'])} summaries, {len(fixture['parse_result'])} stdout texts")


if __name__ == "__main__":
    main()
