"""The drop-in boundary: struct layouts, exported symbols, library loading.
No GPU needed."""
import ctypes as ct
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT
from oracle import oracle as orc
from nova_gb300 import build, _lib
from nova_gb300 import nova_pomdp, nova_pomdp_pbvi, nova_pomdp_perseus, nova_pomdp_alpha_vectors
from nova_gb300 import nova_mdp, nova_mdp_vi, nova_mdp_value_function

# (C type name, ctypes mirror, C field names in order)
STRUCTS = [
    ("POMDP", nova_pomdp.NovaPOMDP, "pomdp/pomdp.h"),
    ("MDP", nova_mdp.NovaMDP, "mdp/mdp.h"),
    ("POMDPAlphaVectors", nova_pomdp_alpha_vectors.NovaPOMDPAlphaVectors, "pomdp/policies/pomdp_alpha_vectors.h"),
    ("MDPValueFunction", nova_mdp_value_function.NovaMDPValueFunction, "mdp/policies/mdp_value_function.h"),
    ("POMDPPBVICPU", nova_pomdp_pbvi.NovaPOMDPPBVICPU, "pomdp/algorithms/pomdp_pbvi_cpu.h"),
    ("POMDPPBVIGPU", nova_pomdp_pbvi.NovaPOMDPPBVIGPU, "pomdp/algorithms/pomdp_pbvi_gpu.h"),
    ("POMDPPerseusCPU", nova_pomdp_perseus.NovaPOMDPPerseusCPU, "pomdp/algorithms/pomdp_perseus_cpu.h"),
    ("MDPVICPU", nova_mdp_vi.NovaMDPValueIterationCPU, "mdp/algorithms/mdp_vi_cpu.h"),
    ("MDPVIGPU", nova_mdp_vi.NovaMDPValueIterationGPU, "mdp/algorithms/mdp_vi_gpu.h"),
]
# C field names where the reference's Python mirror uses other spellings.
C_NAMES = {"Vinitial": "VInitial", "Vprime": "VPrime", "d_Vprime": "d_VPrime"}


def _layout_program(include_dir, cxx):
    lines = ["#include <stdio.h>", "#include <stddef.h>"]
    for _, _, hdr in STRUCTS:
        lines.append("#include <nova/%s>" % hdr)
    if cxx:
        lines.append("using namespace nova;")
    lines.append("int main(void) {")
    for cname, mirror, _ in STRUCTS:
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in mirror._fields_:
            cf = C_NAMES.get(f, f)
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, cf, cname, cf))
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout." + ("cpp" if cxx else "c"))
        exe = os.path.join(d, "layout")
        open(src, "w").write("\n".join(lines))
        cc = "g++" if cxx else "gcc"
        subprocess.run([cc, "-I", include_dir, "-o", exe, src], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return dict(line.rsplit(" ", 1) for line in out.strip().split("\n"))


def _mirror_layout():
    out = {}
    for cname, mirror, _ in STRUCTS:
        out["%s size" % cname] = str(ct.sizeof(mirror))
        for f, _ in mirror._fields_:
            out["%s.%s" % (cname, C_NAMES.get(f, f))] = str(getattr(mirror, f).offset)
    return out


def test_headers_match_ctypes_mirror_c_and_cxx():
    ours_c = _layout_program(os.path.join(ROOT, "include"), cxx=False)
    ours_cxx = _layout_program(os.path.join(ROOT, "include"), cxx=True)
    assert ours_c == ours_cxx == _mirror_layout()


@pytest.mark.skipif(not os.path.isdir(os.path.join(orc.REF_DIR, "include")), reason="reference headers not present")
def test_headers_match_reference_headers():
    ours = _layout_program(os.path.join(ROOT, "include"), cxx=True)
    ref = _layout_program(os.path.join(orc.REF_DIR, "include"), cxx=True)
    assert ours == ref


def test_library_exports_every_declared_entry_point():
    lib = _lib.load()
    declared = build.exported_symbols()
    assert len(declared) >= 70
    missing = [name for name in declared if not hasattr(lib, name)]
    assert missing == []
    # ... and nothing else (the version script keeps internals local)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[2] for l in out.split("\n") if len(l.split()) == 3 and l.split()[1] == "T"}
    assert exported == set(declared)


def test_reference_python_names_are_bound():
    """Every entry point the reference's ctypes modules bind for the hot path
    (python/nova/nova_pomdp_pbvi.py, nova_pomdp_perseus.py, nova_mdp_vi.py,
    nova_mdp.py, nova_pomdp_alpha_vectors.py, nova_mdp_value_function.py)."""
    lib = _lib.load()
    names = []
    for alg in ("pomdp_pbvi", "pomdp_perseus", "mdp_vi"):
        for op in ("initialize", "execute", "uninitialize", "update", "get_policy"):
            for dev in ("cpu", "gpu"):
                names.append("%s_%s_%s" % (alg, op, dev))
    names += ["pomdp_initialize_cpu", "pomdp_uninitialize_cpu", "pomdp_belief_update_cpu",
              "pomdp_add_new_raw_beliefs_cpu", "pomdp_initialize_gpu", "pomdp_uninitialize_gpu",
              "mdp_initialize_cpu", "mdp_uninitialize_cpu", "mdp_initialize_gpu", "mdp_uninitialize_gpu",
              "pomdp_alpha_vectors_initialize", "pomdp_alpha_vectors_value_and_action",
              "pomdp_alpha_vectors_uninitialize", "mdp_value_function_initialize", "mdp_value_function_uninitialize",
              "pomdp_expand_random_cpu", "pomdp_expand_distinct_beliefs_cpu", "pomdp_expand_pema_cpu",
              "pomdp_sigma_cpu", "pomdp_expand_random_gpu"]
    for what in ("successors", "state_transitions", "observation_transitions", "rewards", "nonzero_beliefs",
                 "belief_points"):
        names += ["pomdp_initialize_%s_gpu" % what, "pomdp_uninitialize_%s_gpu" % what]
    for what in ("successors", "state_transitions", "rewards", "goals"):
        names += ["mdp_initialize_%s_gpu" % what, "mdp_uninitialize_%s_gpu" % what]
    assert [n for n in names if not hasattr(lib, n)] == []
