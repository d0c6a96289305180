"""The benchmark's traffic model (CPU): the algorithmic bytes behind `roofline.achieved`
follow the hot-path scope table's formulas and constraint counts for each configuration,
and the per-frame model gives its bytes per particle-iteration."""
import bench


def test_iteration_bytes_follow_the_constraint_counts():
    # 12 C_s + 20 C_b + 12 C_a + 28 N with the table's counts
    small = 12 * 16_002 + 20 * 3_969 + 12 * 8_192 + 28 * 4_096
    large = 12 * 260_610 + 20 * 65_025 + 12 * 131_072 + 28 * 65_536
    assert bench.iteration_bytes(bench.workload("small")) == small
    assert bench.iteration_bytes(bench.workload("large")) == large


def test_recomputed_lra_term_is_left_out_of_the_stress_iteration():
    """1,024 slots exceed the per-particle cache: the kernel recomputes the rests instead of
    streaming C_a = 1.07e9 attachment entries, so C_a is reported apart."""
    stress = 12 * 4_188_162 + 20 * 1_046_529 + 28 * 1_048_576
    assert bench.iteration_bytes(bench.workload("stress")) == stress


def test_frame_model_bytes_per_particle_iteration():
    """With k = 12 cached neighbours: small ~147, large ~134, stress ~125 B per
    particle-iteration (the stress figure without the LRA term)."""
    for name, expect in (("small", 147.0), ("large", 134.0), ("stress", 125.0)):
        wl = bench.workload(name)
        per = bench.frame_bytes(wl, 12.0) / bench.pits_per_frame(wl)
        assert abs(per - expect) / expect < 0.02, (name, per)


def test_batched_workload_is_the_512_cloth_mix():
    wl = bench.workload("batched")
    assert len(wl.cloths) == 512
    assert wl.num_particles == 6_865_422
    assert bench.pits_per_frame(wl) == 6_865_422 * 5 * 10
    assert all(16 <= c.side <= 256 for c in wl.cloths)


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the CPU restatement on the host cores) prints one JSON
    line with the metric, its own CPU baseline and an end-to-end figure without copies."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(bench.__file__).resolve().parent
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         cwd=root, capture_output=True, text=True, timeout=600, check=True).stdout
    line = json.loads(out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["unit"] == "particle-iterations/s" and line["higher_is_better"] is True
    assert line["metric"].startswith("particle-iterations/s")
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
