"""trinkmerd: concurrent clients over a Unix socket get the same files the
drop-in tools write."""
import socket
import subprocess
import threading
import time

import pytest

from trinityrnaseq_gb300.build import BIN
from trinityrnaseq_gb300.kmer import format_histo
from tests.helpers import sort_stats, trinity_r2t_sort

pytestmark = pytest.mark.gpu


def ask(path, line, timeout=120):
    s = socket.socket(socket.AF_UNIX, socket.SOCK_STREAM)
    s.settimeout(timeout)
    s.connect(str(path))
    s.sendall(line.encode() + b"\n")
    out = b""
    while not out.endswith(b"\n"):
        chunk = s.recv(4096)
        if not chunk:
            break
        out += chunk
    s.close()
    return out.decode().strip()


def test_daemon_jobs(native_built, oracle, golden, tmp_path):
    sock = tmp_path / "tk.sock"
    proc = subprocess.Popen([str(BIN / "trinkmerd"), "--socket", str(sock), "--slots", "3", "--budget-gb", "8"],
                            stderr=subprocess.PIPE)
    try:
        for _ in range(200):
            if sock.exists():
                break
            time.sleep(0.05)
        both = tmp_path / "both.fa"
        both.write_bytes((golden / "left.fa").read_bytes() + (golden / "right.fa").read_bytes())
        for n in ("left.fa", "right.fa", "r2t.bundle.fa", "r2t.reads.fa"):
            (tmp_path / n).write_bytes((golden / n).read_bytes())
        reqs = [f"COUNT 25 1 2 {both} {tmp_path}/dump.fa {tmp_path}/dump.histo",
                f"NORMALIZE 25 1 {tmp_path}/left.fa {tmp_path}/right.fa {tmp_path}/l.stats {tmp_path}/r.stats",
                f"R2T 25 0 0 {tmp_path}/r2t.reads.fa {tmp_path}/r2t.bundle.fa {tmp_path}/r2c.out",
                f"SELECT 25 1 3 1 10000 {tmp_path}/left.fa {tmp_path}/right.fa {tmp_path}/l.norm.fa "
                f"{tmp_path}/r.norm.fa {tmp_path}/sel.accs",
                f"COUNT 25 1 1 {tmp_path}/missing.fa {tmp_path}/x.fa"]
        answers = [None] * len(reqs)

        def go(i):
            answers[i] = ask(sock, reqs[i])

        threads = [threading.Thread(target=go, args=(i,)) for i in range(len(reqs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert all(a.startswith("OK") for a in answers[:4]), answers
        assert answers[4].startswith("ERR")
        keys, counts = oracle.count(both.read_bytes(), 25, True)
        assert (tmp_path / "dump.fa").read_bytes() == oracle.dump(keys, counts, 25, 2)
        assert (tmp_path / "dump.histo").read_bytes() == format_histo(oracle.histo(counts), 1, 10000)
        assert sort_stats((tmp_path / "l.stats").read_bytes()) == (golden / "left.stats").read_bytes()
        assert sort_stats((tmp_path / "r.stats").read_bytes()) == (golden / "right.stats").read_bytes()
        assert trinity_r2t_sort((tmp_path / "r2c.out").read_bytes()) == (golden / "r2t.out.sort").read_bytes()
        # the whole normalization: nbkc_normalize.pl's accs (the reference scripts' own output) and the
        # records they select
        accs = (tmp_path / "sel.accs").read_bytes()
        assert accs == (golden / "normalized.accs").read_bytes()
        for side in ("left", "right"):
            assert (tmp_path / f"{side[0]}.norm.fa").read_bytes() == \
                oracle.norm_extract((golden / f"{side}.fa").read_bytes(), accs)
        st = ask(sock, "STATS").split()
        assert st[0] == "OK" and int(st[1]) == 4
        assert ask(sock, "QUIT") == "OK"
        assert proc.wait(timeout=60) == 0
    finally:
        if proc.poll() is None:
            proc.kill()
            proc.wait()
