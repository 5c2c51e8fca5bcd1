"""The autotuner's search space and its record (no GPU needed): the split
density scan's bit is swept only where it can apply, the Python limit is the
library's, and the recorded choices are valid variants."""
import json
import os
import re

from libfluid_gb300 import autotune

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _define(path: str, name: str) -> int:
    text = open(os.path.join(ROOT, path)).read()
    m = re.search(r"#define\s+" + name + r"\s+(0x[0-9a-fA-F]+|\d+)u?", text)
    assert m, name
    return int(m.group(1), 0)


def test_split_limit_matches_the_library():
    assert autotune.DENSITY_SPLIT_MAX == _define("libfluid_gb300/csrc/sph_types.h", "SPH_DENSITY_SPLIT_MAX")
    assert _define("include/sph_c.h", "SPH_VARIANT_DENSITY_SPLIT") == 0x20
    assert _define("libfluid_gb300/csrc/sph_types.h", "SPH_VARIANT_MASK") == len(autotune.VARIANTS) - 1


def test_split_bit_swept_only_where_it_applies():
    small = autotune.variants_for(autotune.DENSITY_SPLIT_MAX, 0)
    assert small == tuple(range(64))
    assert autotune.variants_for(autotune.DENSITY_SPLIT_MAX + 1, 0) == tuple(range(32))
    assert autotune.variants_for(32768, 2) == tuple(range(32))   # persistent tiles: no split scan


def test_tuned_record_is_valid():
    tuned = json.load(open(os.path.join(ROOT, "libfluid_gb300", "tuned.json")))
    mask = _define("libfluid_gb300/csrc/sph_types.h", "SPH_VARIANT_MASK")
    for name, rec in tuned.items():
        best = rec["best"]
        assert best["tile"] in (64, 128, 256), name
        assert 0 < best["skin"] <= 1, name
        assert best["variant"] & ~mask == 0, name
        if rec["particles"] > autotune.DENSITY_SPLIT_MAX:
            assert all(t["variant"] < 32 for t in rec["trials"]), name
    # the 32,768-particle scene's sweep covered the split bit and chose it
    small = tuned["small_dam_break"]
    assert any(t["variant"] & 0x20 for t in small["trials"])
    assert small["best"]["variant"] & 0x20
