"""Command-line checks of bin/insilico_read_normalization that stop the run
before any GPU work (the script's own checks, util/insilico_read_normalization.pl:
184-250), so they run without a GPU."""
import subprocess

import pytest

from trinityrnaseq_gb300.build import BIN


def run(args, tmp_path):
    return subprocess.run([str(BIN / "insilico_read_normalization"), *map(str, args)], cwd=tmp_path,
                          capture_output=True, text=True, timeout=60)


BASE = ["--seqType", "fq", "--JM", "10G", "--max_cov", 200, "--left", "l.fq", "--right", "r.fq", "--pairs_together"]


@pytest.mark.parametrize("change,message", [
    ({"--seqType": "fastq"}, "set --seqType to 'fq' or 'fa'"),
    ({"--JM": "10"}, "must set --JM"),
    ({"--JM": "G"}, "must set --JM"),
    ({"--max_cov": 1}, "--max_cov at least 2"),
    ({"--SS_lib_type": "XY"}, "unrecognized SS_lib_type"),
])
def test_option_checks(native_built, tmp_path, change, message):
    args = list(BASE)
    for k, v in change.items():
        if k in args:
            args[args.index(k) + 1] = v
        else:
            args += [k, v]
    p = run(args, tmp_path)
    assert p.returncode != 0 and message in p.stderr, p.stderr


def test_reads_required(native_built, tmp_path):
    p = run(["--seqType", "fq", "--JM", "10G", "--max_cov", 200], tmp_path)
    assert p.returncode != 0 and "need either options 'left' and 'right' or option 'single'" in p.stderr


def test_pairs_together_needs_pairs(native_built, tmp_path):
    p = run(["--seqType", "fq", "--JM", "10G", "--max_cov", 200, "--single", "s.fq", "--pairs_together"], tmp_path)
    assert p.returncode != 0 and "--pairs_together" in p.stderr


def test_reverse_complemented_fasta_refused(native_built, tmp_path):
    p = run(["--seqType", "fa", "--JM", "10G", "--max_cov", 200, "--left", "l.fa", "--right", "r.fa",
             "--SS_lib_type", "RF"], tmp_path)
    assert p.returncode != 0 and "not provided" in p.stderr


def test_unknown_option(native_built, tmp_path):
    p = run(BASE + ["--bogus"], tmp_path)
    assert p.returncode != 0 and "do not understand option" in p.stderr
