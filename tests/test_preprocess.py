"""Host side of the preprocessing row (no GPU): CSV reading, date alignment
and split against the oracle's plain-Python restatement of
preprocessing/fetch_split.py:86-124, and the .bin layout of
preprocessing/save_binary.py:23-45 / src/utilities/load_binary.c."""
import datetime as dt
import os

import numpy as np
import pytest

from riskgpu import preprocess


def write_index_files(directory, seed=7, n_idx=5, days=400):
    """Seeded synthetic index files in the reference's layout: 'Date'
    (m/d/Y, newest first) and 'Return' (4 decimals); each index misses some
    dates, one row has an unparseable date and one a missing return."""
    rng = np.random.default_rng(seed)
    start = dt.date(2016, 1, 4)
    all_days = [start + dt.timedelta(days=i) for i in range(days)]
    series = {}
    files = {}
    for j in range(n_idx):
        keep = rng.random(days) > 0.05
        rows = []
        for d, kept in zip(all_days, keep):
            if kept:
                r = round(float(rng.normal(3e-4, 0.012)), 4)
                rows.append((d, r))
        name, fname = f"IDX{j}", f"idx{j}.csv"
        with open(os.path.join(directory, fname), "w") as f:
            f.write("Date,Return\n")
            for i, (d, r) in enumerate(reversed(rows)):
                if j == 1 and i == 3:
                    f.write(f"{d.month}/{d.day}/{d.year},\n")       # missing return
                    rows[len(rows) - 1 - i] = (d, None)
                    continue
                f.write(f"{d.month:02d}/{d.day:02d}/{d.year},{r:.4f}\n")
            if j == 0:
                f.write("not-a-date,0.0100\n")
        series[name] = rows
        files[name] = fname
    return files, series


def test_fetch_and_split_matches_the_oracle(tmp_path, oracle):
    files, series = write_index_files(str(tmp_path))
    files_with_missing = dict(files, GHOST="ghost.csv")          # skipped, as the reference skips it
    start, end = dt.date(2016, 2, 1), dt.date(2016, 12, 31)
    train, test = preprocess.fetch_and_split(files_with_missing, str(tmp_path), start=str(start), end=str(end),
                                             train_ratio=0.7)
    ref_train, ref_test = oracle.align_and_split(series, start, end, 0.7)
    for got, ref in ((train, ref_train), (test, ref_test)):
        assert len(got) == len(ref)
        assert [np.datetime64(d, "D") for d, _ in ref] == list(got.dates)
        assert np.array_equal(np.array([v for _, v in ref], dtype=np.float64), got.values)
    assert train.names == list(files)
    assert (np.diff(train.dates.astype(np.int64)) > 0).all()


def test_fetch_and_split_errors(tmp_path):
    files, _ = write_index_files(str(tmp_path), days=90)
    with pytest.raises(ValueError, match="insufficient"):
        preprocess.fetch_and_split(files, str(tmp_path), start="2016-01-01", end="2017-01-01")
    with pytest.raises(ValueError, match="no index file"):
        preprocess.fetch_and_split({"A": "none.csv"}, str(tmp_path))
    files, _ = write_index_files(str(tmp_path), days=300)
    with pytest.raises(ValueError, match="train_ratio"):
        preprocess.fetch_and_split(files, str(tmp_path), start="2016-01-01", end="2017-01-01", train_ratio=1.0)
    with pytest.raises(ValueError, match="no data"):
        preprocess.fetch_and_split(files, str(tmp_path), start="2030-01-01", end="2031-01-01")


def test_binary_layout_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    mu = rng.normal(size=7)
    a = rng.normal(size=(7, 7))
    sigma = a @ a.T
    preprocess.save_results_binary(mu, sigma, 0.0123, str(tmp_path))
    raw = open(os.path.join(tmp_path, "mu.bin"), "rb").read()
    assert np.frombuffer(raw[:4], dtype=np.int32)[0] == 7 and len(raw) == 4 + 8 * 7
    raw = open(os.path.join(tmp_path, "sigma.bin"), "rb").read()
    assert list(np.frombuffer(raw[:8], dtype=np.int32)) == [7, 7] and len(raw) == 8 + 8 * 49
    assert len(open(os.path.join(tmp_path, "params.bin"), "rb").read()) == 8
    m2, s2, f2 = preprocess.load_results_binary(str(tmp_path))
    assert np.array_equal(m2, mu) and np.array_equal(s2, sigma) and f2 == 0.0123


REFERENCE_TREE = "/root/reference"


def _reference_config():
    """The index files and parameters of the reference's config.yaml, read
    as text (PyYAML is not assumed): indices, start, end, train_ratio, x, k."""
    path = os.path.join(REFERENCE_TREE, "config.yaml")
    indices, cfg, in_idx = {}, {}, False
    for line in open(path):
        text = line.split("#", 1)[0].rstrip()
        if not text.strip():
            continue
        if not line.startswith(" "):
            in_idx = text.startswith("indices:")
            if ":" in text and not in_idx:
                key, val = text.split(":", 1)
                cfg[key.strip()] = val.strip().strip('"')
            continue
        if in_idx and ":" in text:
            key, val = text.split(":", 1)
            indices[key.strip()] = val.strip().strip('"')
    return indices, cfg


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE_TREE, "dataset")),
                    reason="the reference's index files are not on this machine")
def test_reference_dataset_split_matches_the_oracle(oracle):
    """The reference's own index files and config.yaml (15 indices, daily
    returns since 2015, 80/20 split): the engine's reader, alignment and split
    against the oracle's plain-Python restatement, row by row, and the
    training moments and realised crash frequency against the oracle's."""
    import csv
    import math
    indices, cfg = _reference_config()
    assert len(indices) >= 5
    dataset = os.path.join(REFERENCE_TREE, "dataset")
    start, end = cfg["start"], cfg["end"]
    ratio, x, k = float(cfg["train_ratio"]), float(cfg["x"]), int(cfg["k"])
    train, test = preprocess.fetch_and_split(indices, dataset, start=start, end=end, train_ratio=ratio)

    series = {}
    for name, fname in indices.items():
        rows = []
        with open(os.path.join(dataset, fname), newline="") as f:
            for row in csv.DictReader(f):
                try:
                    d = dt.datetime.strptime(row["Date"].strip(), "%m/%d/%Y").date()
                except ValueError:
                    continue
                try:
                    r = float(row["Return"])
                except (TypeError, ValueError):
                    r = None
                rows.append((d, None if r is None or math.isnan(r) else r))
        series[name] = rows
    to_date = lambda s: dt.date.fromisoformat(s)
    ref_train, ref_test = oracle.align_and_split(series, to_date(start), to_date(end), ratio)
    for got, ref in ((train, ref_train), (test, ref_test)):
        assert len(got) == len(ref) and len(got) > 100
        assert [np.datetime64(d, "D") for d, _ in ref] == list(got.dates)
        assert np.array_equal(np.array([v for _, v in ref], dtype=np.float64), got.values)
    assert train.names == list(indices)
    assert train.dates[-1] < test.dates[0]
    mu, sigma = oracle.compute_stats(train.values)
    assert mu.shape == (len(indices),) and np.all(np.linalg.eigvalsh(sigma) > 0)
    freq = oracle.compute_metrics(test.values, x, k)
    assert 0.0 <= freq <= 1.0
