"""Synthetic dbgen-layout .tbl files for the loader tests: random rows of our
own in the column layout of lineitem and part (fields separated and rows
ended by '|'); no TPC-H rows or answers."""
import datetime

import numpy as np

EPOCH = datetime.date(1970, 1, 1)


def write_tables(tmp_path, n_part=500, n_lineitem=4000, seed=1):
    rng = np.random.default_rng(seed)
    partkey = np.arange(1, n_part + 1, dtype=np.uint64)
    promo = (rng.random(n_part) < 0.2).astype(np.uint8)
    with open(tmp_path / "part.tbl", "w") as f:
        for k, p in zip(partkey, promo):
            kind = "PROMO synthetic" if p else ("PROM synthetic" if k % 7 == 0 else "OTHER synthetic")
            f.write(f"{k}|name {k}|m|b|{kind}|{int(k) % 50}|c|{900 + int(k) % 100}.{int(k) % 100:02d}|x|\n")
    l_partkey = rng.integers(1, n_part + 60, n_lineitem).astype(np.uint32)  # some without a part
    base = (datetime.date(1995, 8, 1) - EPOCH).days
    l_ship = (base + rng.integers(0, 92, n_lineitem)).astype(np.uint32)     # around the Q14 month
    price = rng.integers(90000, 10500000, n_lineitem).astype(np.int64)    # cents
    disc = rng.integers(0, 11, n_lineitem).astype(np.int64)               # hundredths
    with open(tmp_path / "lineitem.tbl", "w") as f:
        for i in range(n_lineitem):
            ship = EPOCH + datetime.timedelta(days=int(l_ship[i]))
            f.write(f"{i // 4 + 1}|{l_partkey[i]}|{i % 97}|{i % 4 + 1}|{i % 50 + 1}|"
                    f"{price[i] // 100}.{price[i] % 100:02d}|0.{disc[i]:02d}|0.0{i % 9}|A|B|"
                    f"{ship.isoformat()}|{ship.isoformat()}|{ship.isoformat()}|s|m|comment {i}|\n")
    cols = {"l_partkey": l_partkey, "l_shipdate": l_ship, "l_extendedprice": price, "l_discount": disc,
            "p_partkey": partkey, "p_promo": promo}
    return str(tmp_path / "lineitem.tbl"), str(tmp_path / "part.tbl"), cols


def q14_sums(cols):
    lo = (datetime.date(1995, 9, 1) - EPOCH).days
    hi = (datetime.date(1995, 10, 1) - EPOCH).days
    promo = dict(zip(cols["p_partkey"].tolist(), cols["p_promo"].tolist()))
    s_promo = s_all = 0
    for pk, d, p, dc in zip(cols["l_partkey"].tolist(), cols["l_shipdate"].tolist(),
                            cols["l_extendedprice"].tolist(), cols["l_discount"].tolist()):
        if lo <= d < hi and pk in promo:
            v = p * (100 - dc)
            s_all += v
            if promo[pk]:
                s_promo += v
    return s_promo, s_all
