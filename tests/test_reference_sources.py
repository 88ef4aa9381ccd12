"""The reference checker's sources are the reference's own files, copied unchanged (CPU)."""
import hashlib
import json
import os

import pytest

from oracle import ref_build


def test_checker_sources_are_unchanged_copies():
    if not ref_build.sources_present():
        pytest.skip("no reference checkout was available to copy from")
    rec = json.load(open(os.path.join(ref_build.SRC, "SHA256.json")))
    for f in ref_build.FILES:
        dst = os.path.join(ref_build.SRC, f)
        assert hashlib.sha256(open(dst, "rb").read()).hexdigest() == rec[f]
        src = os.path.join(ref_build.REF, f)
        if os.path.exists(src):
            assert open(src, "rb").read() == open(dst, "rb").read()


def test_stand_in_headers_declare_the_reference_globals():
    src = open(os.path.join(ref_build.STUBS, "cpuEvaluator.h")).read()
    for g in ("extern int layers;", "extern std::vector<float> z_layers;", "extern std::vector<int> waves_begin;",
              "extern std::vector<int> waves_end;", "extern std::vector<UnpackedWave<float>> W;"):
        assert g in src
