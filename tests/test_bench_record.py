"""bench.py's ncu record lookup: traffic and pipe figures are taken from a
profile summary's `bench-record:` line only when the line names the running
build's digest, the kernel and the resolution; otherwise the bench reports
traffic as unmeasured.  Also checks that the committed step-1 record parses."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402

LINE = ("bench-record: digest=0123456789abcdef kernel=k_de_grid_brick res=512 "
        "dram_bytes=622720256 fma=60.49 alu=22.45 xu=13.30 issue=87.80\n")


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_record_found_for_its_digest(tmp_path):
    write(tmp_path, "k.md", "# profile\n\n" + LINE)
    rec = bench.ncu_record("k_de_grid_brick", 512, pdir=str(tmp_path),
                           digest="0123456789abcdef" + "0" * 48)
    assert rec is not None
    assert int(rec["dram_bytes"]) == 622720256 and float(rec["issue"]) == 87.80


def test_record_of_another_build_kernel_or_size_is_ignored(tmp_path):
    write(tmp_path, "k.md", LINE)
    assert bench.ncu_record("k_de_grid_brick", 512, pdir=str(tmp_path),
                            digest="fedcba9876543210") is None
    assert bench.ncu_record("k_de_grid", 512, pdir=str(tmp_path),
                            digest="0123456789abcdef") is None
    assert bench.ncu_record("k_de_grid_brick", 256, pdir=str(tmp_path),
                            digest="0123456789abcdef") is None


def test_only_markdown_summaries_are_read(tmp_path):
    write(tmp_path, "k.txt", LINE)
    assert bench.ncu_record("k_de_grid_brick", 512, pdir=str(tmp_path),
                            digest="0123456789abcdef") is None
    assert bench.ncu_record("k_de_grid_brick", 512, pdir=str(tmp_path / "missing"),
                            digest="0123456789abcdef") is None


def test_committed_step1_record_parses():
    """The committed summary holds one record for the step-1 kernel at res
    512, with every field the bench reads."""
    path = os.path.join(ROOT, "profiles", "k_de_grid_brick_res512.md")
    lines = [l for l in open(path) if l.startswith("bench-record:")]
    assert len(lines) == 1
    digest = lines[0].split("digest=", 1)[1].split()[0]
    assert len(digest) == 16 and all(c in "0123456789abcdef" for c in digest)
    rec = bench.ncu_record("k_de_grid_brick", 512, digest=digest)
    assert rec is not None
    for k in ("dram_bytes", "fma", "alu", "xu", "issue"):
        float(rec[k])
