"""bench.py's DRAM traffic record (CPU): an ncu launch list becomes per-kernel DRAM bytes
per launch of the variant the run settled on, tagged with the kernel sources' hash; the
headline's roofline reads it only while the sources are unchanged."""

import csv
import json

import bench

HEAD = ["ID", "Process ID", "Process Name", "Host Name", "Kernel Name", "Context", "Stream", "Block Size",
        "Grid Size", "Device", "CC", "Section Name", "Metric Name", "Metric Unit", "Metric Value"]


def _rows(lid, name, rd, wr, ns):
    base = [str(lid), "1", "python", "h", name, "1", "7", "(256, 1, 1)", "(4128, 1, 1)", "0", "10.3", "Command line"]
    return [base + ["dram__bytes_read.sum", "byte", f"{rd:,}"],
            base + ["dram__bytes_write.sum", "Mbyte", str(wr / 1e6)],
            base + ["gpu__time_duration.sum", "nsecond", f"{ns:,}"]]


def test_record_keeps_the_last_variant_per_kind_and_checks_the_source_hash(tmp_path, monkeypatch):
    rows = [["==PROF== Connected to process"], HEAD]
    # the autotuner first times the persistent x inverse, the run then settles on the
    # one-tile one; a y-pass name carries parentheses inside its template arguments
    rows += _rows(1, "void l3es::kx_inv_tma<256, 1, 1, 1>(CUtensorMap_st, float2 *)", 100, 200e6, 130000)
    rows += _rows(2, "void l3es::kx_inv<256, 3, 1, 1, 1, 8>(const float2 *, long)", 200e6, 300e6, 110000)
    rows += _rows(3, "void l3es::kx_inv<256, 3, 1, 1, 1, 8>(const float2 *, long)", 220e6, 320e6, 112000)
    rows += _rows(4, "void l3es::ky_pass<256, (int)-1, 0>(float2 *, long, int, int, int, const float2 *)",
                  150e6, 30e6, 40000)
    rows += _rows(5, "void l3es::k_crop<3>(const float2 *)", 1e6, 1e6, 5000)
    src = tmp_path / "launches.csv"
    with open(src, "w", newline="") as f:
        csv.writer(f).writerows(rows)
    out = tmp_path / "rec.json"
    rec = bench.record_traffic(str(src), str(out), "ncu ...")
    k = rec["kernels"]
    assert set(k) == {"kx_inv_curl", "ky_pass_fwd"}
    assert k["kx_inv_curl"]["kernel"] == "kx_inv<256, 3, 1, 1, 1, 8>"
    assert k["kx_inv_curl"]["launches"] == 2
    assert abs(k["kx_inv_curl"]["traffic_per_launch"] - (420e6 + 620e6) / 2) < 1.0
    assert abs(k["kx_inv_curl"]["us_per_launch_serialised"] - 111.0) < 1e-9
    assert k["ky_pass_fwd"]["kernel"] == "ky_pass<256, (int)-1, 0>"
    assert json.load(open(out))["sources_sha256"] == bench.sources_sha256()
    # the roofline reads the record for these sources, and refuses it for others
    monkeypatch.setattr(bench, "TRAFFIC_JSON", str(out))
    traffic, why = bench._ncu_traffic("kx_inv_curl")
    assert traffic == k["kx_inv_curl"]["traffic_per_launch"] and "ncu" in why
    assert bench._ncu_traffic("line_cross")[0] is None
    monkeypatch.setattr(bench, "sources_sha256", lambda: "0" * 64)
    traffic, why = bench._ncu_traffic("kx_inv_curl")
    assert traffic is None and "other kernel sources" in why
