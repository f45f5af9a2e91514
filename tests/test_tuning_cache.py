"""The subdomain-count cache that bench.py and callers read
(rchol_gb300/tuning.py): keys by matrix shape and precision, the default
when a shape is absent or the file is missing or unreadable, and the
committed entry for the bench's own matrix (256^3 log-normal 7-point
Laplacian, FP32 G), whose chosen count must be a power of two that the
ordering accepts and the fastest of the timed candidates."""

import json

import rchol_gb300 as R
from rchol_gb300 import tuning


def test_lookup_default_and_precision(tmp_path):
    path = tmp_path / "cache.json"
    assert tuning.subdomains_for(1000, 7000, path=str(path)) == 2048  # no file
    path.write_text("not json")
    assert tuning.subdomains_for(1000, 7000, default=64, path=str(path)) == 64  # unreadable file
    cache = {tuning._key(1000, 7000, R.PREC_FP32): {"subdomains": 16}}
    path.write_text(json.dumps(cache))
    assert tuning.subdomains_for(1000, 7000, R.PREC_FP32, path=str(path)) == 16
    assert tuning.subdomains_for(1000, 7000, R.PREC_FP64, path=str(path)) == 2048  # other precision
    assert tuning.subdomains_for(1000, 7001, R.PREC_FP32, path=str(path)) == 2048  # other shape


def test_committed_entry_for_the_bench_matrix():
    n, nnz = 256 ** 3, 117047296  # generators.laplace_3d_weighted(256, 1.0, 1e-3, 0)
    ent = tuning.load_cache().get(tuning._key(n, nnz, R.PREC_FP32))
    assert ent is not None
    t = int(ent["subdomains"])
    assert t > 0 and t & (t - 1) == 0
    timed = {int(k): v["ms"] for k, v in ent["results"].items()}
    assert t == min(timed, key=timed.get)
    assert tuning.subdomains_for(n, nnz, R.PREC_FP32) == t
