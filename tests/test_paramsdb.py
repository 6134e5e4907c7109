"""ParamsDB request source on CPU: the reference's HParams.db table layout
(src/inc/DB.h:31-33), insert-or-update by name, fetch, and an unknown name."""
import sqlite3

import numpy as np
import pytest

from hestonexotics_gb300 import engine as E
from hestonexotics_gb300.paramsdb import NotFound, ParamsDB


def test_roundtrip_and_schema(tmp_path):
    path = tmp_path / "HParams.db"
    with ParamsDB(path) as db:
        db.insertupdate(E.Params(0.04, 0.05, -0.7, 1.5, 0.5), "SPY")
        db.insertupdate(E.Params(0.09, 0.09, 0.04, 1.0, 1.0), "QQQ")
        db.insertupdate(E.Params(0.03, 0.05, -0.6, 2.0, 0.4), "SPY")   # update in place
        assert db.names() == ["QQQ", "SPY"]
        p = db.fetch("SPY", r=0.02)
        assert (p.v0, p.theta, p.rho, p.kappa, p.sigma, p.r) == (0.03, 0.05, -0.6, 2.0, 0.4, 0.02)
        with pytest.raises(NotFound):
            db.fetch("IWM")
        rq = db.request("QQQ", 100.0, E.Options(np.array([100.0]), np.array([1.0]), E.ASIAN), seed=7)
        assert rq.params.v0 == 0.09 and rq.seed == 7
    # the column layout the reference's ParamsDB::fetch reads by position (DB.h:34-42)
    con = sqlite3.connect(str(path))
    cols = [r[1] for r in con.execute("PRAGMA table_info(HestonParameters)")]
    assert cols == ["Name", "V0", "Vm", "Rho", "Kappa", "Sigma", "ComputedAt"]
    row = con.execute("SELECT * FROM HestonParameters WHERE Name='SPY'").fetchone()
    assert row[1:6] == (0.03, 0.05, -0.6, 2.0, 0.4) and row[6] > 0
