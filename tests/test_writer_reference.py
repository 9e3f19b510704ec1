"""The spectrum writer's layout against the reference's own writer: the
datasets pbag::writer_datasets lists for a layer group (include/
pbag_recorder.hpp) must be, for every combination of the options that gate
them (numeric electrons, SSA, SSC, reverse-shock radiation), the datasets
Ejecta::computeSaveEjectaSpectrum stores (ejecta.h:354-455), in its order.
The reference sequence is read from the writer's source: every
Output::addVectorToGroup call with the options of the `if` blocks around it."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("PBAG_REF_SRC") or os.path.join(os.path.dirname(ROOT), "reference", "src")
EJECTA_H = os.path.join(REF_SRC, "ejecta", "ejecta.h")

GUARDS = (("m_eleMethod", "ele"), ("m_methods_ssa", "ssa"), ("m_methods_ssc", "ssc"),
          ("do_rs_radiation", "rs"))


def reference_sequence():
    """[(dataset name, {options that gate it})] of the writer, in order."""
    src = open(EJECTA_H).read()
    start = src.index("void computeSaveEjectaSpectrum(")
    body = src[start:src.index("grp.close();", start)]
    body = re.sub(r"//[^\n]*", "", body)  # comments
    seq, stack, depth, pending = [], [], 0, None
    # statements split at ';', '{' and '}' (the writer's if blocks and calls)
    for tok in re.split(r"(;|\{|\})", body):
        if tok == "{":
            depth += 1
            stack.append((depth, pending))
            pending = None
            continue
        if tok == "}":
            while stack and stack[-1][0] == depth:
                stack.pop()
            depth -= 1
            continue
        if tok == ";":
            continue
        text = " ".join(tok.split())
        guard, is_if = None, text.startswith("if")
        if is_if:  # the condition runs to its matching parenthesis
            i, level = text.index("("), 0
            for k in range(i, len(text)):
                level += {"(": 1, ")": -1}.get(text[k], 0)
                if level == 0:
                    break
            guard = next((g for key, g in GUARDS if key in text[i:k + 1]), None)
            text = text[k + 1:].strip()
        call = re.search(r'Output::addVectorToGroup\(.*"(\w+)"\s*\)$', text)
        active = {g for _, g in stack if g} | ({guard} if guard else set())
        if call:
            seq.append((call.group(1), active))
        elif is_if and not text:
            pending = guard  # an if whose block opens next
    return seq


@pytest.mark.skipif(not os.path.exists(EJECTA_H), reason="reference sources not available")
def test_writer_datasets_follow_reference_writer(tmp_path):
    seq = reference_sequence()
    names = [n for n, _ in seq]
    assert names[:4] == ["n_ele_fs", "gam_dot_syn_fs", "gam_dot_adi_fs", "gam_dot_ssc_fs"], names
    assert len(names) == 30 and names[-1] == "total_a_rs", names
    exe = tmp_path / "writer_names"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "writer_names.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    lines = dict(l.split(":", 1) for l in out.strip().splitlines())
    assert len(lines) == 16
    for key, got in lines.items():
        ele, ssa, ssc, rs = (bool(int(x)) for x in key.split())
        on = {"ele": ele, "ssa": ssa, "ssc": ssc, "rs": rs}
        expect = [n for n, guards in seq if all(on[g] for g in guards)]
        assert got.split() == expect, (key, got.split(), expect)
