"""Market data -> (mu, Sigma, realised crash frequency), with the moments
and the crash count on the GPU.

Host side of the reference's offline pipeline (preprocessing/main.py:8-52),
restated with numpy and the standard library (pandas is not required):

  read_index_csv      one index file: 'Date' (m/d/Y) and 'Return' columns
                      (fetch_split.py:46-63; rows with an unparseable date are
                      dropped, like pd.to_datetime(errors='coerce') + dropna)
  fetch_and_split     union of the indices' dates, ascending (pd.DataFrame of
                      Series, :86); rows in [start, end] inclusive (.loc, :94);
                      rows with any missing return dropped (dropna, :104);
                      at least 100 rows; split at int(rows * train_ratio)
                      (:122-124)
  compute_stats       rg_moments on the GPU (preprocessing_stats.py:18,21)
  compute_metrics     rg_crash_frequency on the GPU (evaluation.py:19,22)
  save_results_binary mu.bin / sigma.bin / params.bin (save_binary.py:23-45)
  run_pipeline        the four steps in order (main.py:30-43), from a config
                      dict with the keys of the reference's config.yaml
"""
from __future__ import annotations

import csv
import datetime as _dt
import os
from dataclasses import dataclass

import numpy as np

from . import crash_frequency, moments


@dataclass
class Returns:
    """Aligned daily returns: dates ascending, one column per index."""
    dates: np.ndarray      # datetime64[D], shape (T,)
    names: list            # index names, column order
    values: np.ndarray     # float64, shape (T, N)

    def __len__(self):
        return len(self.dates)


def _parse_date(text: str):
    try:
        return np.datetime64(_dt.datetime.strptime(text.strip(), "%m/%d/%Y").date(), "D")
    except (ValueError, AttributeError):
        return None


def _parse_float(text: str) -> float:
    try:
        return float(text)
    except (TypeError, ValueError):
        return float("nan")


def read_index_csv(path: str):
    """(dates, returns) of one index file; rows whose date does not parse as
    m/d/Y are dropped; a return that does not parse is NaN."""
    dates, rets = [], []
    with open(path, newline="") as f:
        reader = csv.DictReader(f)
        if reader.fieldnames is None or "Date" not in reader.fieldnames or "Return" not in reader.fieldnames:
            raise ValueError(f"{path}: missing 'Date' or 'Return' column")
        for row in reader:
            d = _parse_date(row.get("Date") or "")
            if d is None:
                continue
            dates.append(d)
            rets.append(_parse_float(row.get("Return")))
    return np.array(dates, dtype="datetime64[D]"), np.array(rets, dtype=np.float64)


def _to_day(value) -> np.datetime64:
    if isinstance(value, np.datetime64):
        return value.astype("datetime64[D]")
    return np.datetime64(str(value), "D")


def align(series: dict) -> Returns:
    """Union of the dates of every index (ascending); a date an index lacks
    holds NaN for it."""
    names = list(series.keys())
    all_dates = np.unique(np.concatenate([series[k][0] for k in names])) if names else np.array([], "datetime64[D]")
    values = np.full((len(all_dates), len(names)), np.nan)
    for j, k in enumerate(names):
        d, r = series[k]
        if len(np.unique(d)) != len(d):
            raise ValueError(f"index {k}: duplicate dates")
        values[np.searchsorted(all_dates, d), j] = r
    return Returns(all_dates, names, values)


def fetch_and_split(indices: dict, dataset_dir: str, start="2015-01-01", end="2025-01-01", train_ratio=0.7):
    """(train, test) Returns from the index CSV files named by `indices`
    (index name -> file name under dataset_dir).  Missing or malformed files
    are skipped, as the reference skips them; no file at all is an error."""
    series = {}
    for name, filename in indices.items():
        path = os.path.join(dataset_dir, filename)
        if not os.path.exists(path):
            continue
        try:
            series[name] = read_index_csv(path)
        except (ValueError, OSError):
            continue
    if not series:
        raise ValueError("no index file could be loaded")
    ret = align(series)
    lo, hi = _to_day(start), _to_day(end)
    keep = (ret.dates >= lo) & (ret.dates <= hi)
    ret = Returns(ret.dates[keep], ret.names, ret.values[keep])
    if len(ret) == 0:
        raise ValueError(f"no data in the date range {start} to {end}")
    full = ~np.isnan(ret.values).any(axis=1)
    ret = Returns(ret.dates[full], ret.names, ret.values[full])
    if len(ret) < 100:
        raise ValueError(f"insufficient data: {len(ret)} days after alignment (at least 100 needed)")
    if not 0.0 < train_ratio < 1.0:
        raise ValueError(f"train_ratio must be in (0, 1), got {train_ratio}")
    split = int(len(ret) * train_ratio)
    train = Returns(ret.dates[:split], ret.names, ret.values[:split])
    test = Returns(ret.dates[split:], ret.names, ret.values[split:])
    return train, test


def compute_stats(train: Returns):
    """(mu, Sigma) of the training returns, on the GPU."""
    return moments(train.values)


def compute_metrics(test: Returns, x=0.02, k=5) -> float:
    """Realised frequency of days with at least k indices below -x, on the GPU."""
    return crash_frequency(test.values, x, k)


def save_results_binary(mu, sigma, actual_freq, output_dir) -> None:
    """mu.bin: int32 N + N f64; sigma.bin: int32 rows, int32 cols + row-major
    f64; params.bin: one f64 (the layout load_binary.c reads)."""
    os.makedirs(output_dir, exist_ok=True)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    with open(os.path.join(output_dir, "mu.bin"), "wb") as f:
        f.write(np.int32(mu.shape[0]).tobytes())
        f.write(mu.tobytes())
    with open(os.path.join(output_dir, "sigma.bin"), "wb") as f:
        f.write(np.array(sigma.shape, dtype=np.int32).tobytes())
        f.write(sigma.tobytes())
    with open(os.path.join(output_dir, "params.bin"), "wb") as f:
        f.write(np.float64(actual_freq).tobytes())


def load_results_binary(directory: str):
    """(mu, Sigma, actual_freq) read back from the three .bin files."""
    with open(os.path.join(directory, "mu.bin"), "rb") as f:
        n = int(np.frombuffer(f.read(4), dtype=np.int32)[0])
        mu = np.frombuffer(f.read(8 * n), dtype=np.float64).copy()
    with open(os.path.join(directory, "sigma.bin"), "rb") as f:
        r, c = (int(v) for v in np.frombuffer(f.read(8), dtype=np.int32))
        sigma = np.frombuffer(f.read(8 * r * c), dtype=np.float64).reshape(r, c).copy()
    with open(os.path.join(directory, "params.bin"), "rb") as f:
        freq = float(np.frombuffer(f.read(8), dtype=np.float64)[0])
    return mu, sigma, freq


def run_pipeline(config: dict, dataset_dir: str, output_dir: str) -> dict:
    """The reference pipeline from a dict with the config.yaml keys
    start, end, x, k, train_ratio and indices (name -> CSV file name)."""
    indices = config["indices"]
    if not isinstance(indices, dict):
        raise TypeError("'indices' must map index names to CSV file names")
    train, test = fetch_and_split(indices, dataset_dir, start=config["start"], end=config["end"],
                                  train_ratio=config["train_ratio"])
    mu, sigma = compute_stats(train)
    actual_freq = compute_metrics(test, x=config["x"], k=config["k"])
    save_results_binary(mu, sigma, actual_freq, output_dir)
    return {"mu": mu, "Sigma": sigma, "actual_freq": actual_freq, "train": train, "test": test}
