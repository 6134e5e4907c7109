"""ParamsDB request source: calibrated Heston parameter sets by name.

The reference keeps calibrated parameters in an SQLite file, HParams.db, one
row per underlying (src/inc/DB.h:31-41, src/DB.cpp:7-39):

    HestonParameters(Name TEXT UNIQUE, V0, Vm, Rho, Kappa, Sigma REAL,
                     ComputedAt INTEGER)

``ParamsDB`` reads and writes the same table with Python's sqlite3 module,
so a database written by the reference serves requests here and the other
way round.  ``request`` turns a row plus an option list into a pricing
request for ``Engine.price_batch`` or the continuous-batching ``Server``.
"""
from __future__ import annotations

import sqlite3
from pathlib import Path

from .engine import Options, Params, Request

CREATE_TABLE = ("CREATE TABLE IF NOT EXISTS HestonParameters (Name TEXT NOT NULL UNIQUE, V0 REAL NOT NULL, "
                "Vm REAL NOT NULL, Rho REAL NOT NULL, Kappa REAL NOT NULL, Sigma REAL NOT NULL, "
                "ComputedAt INTEGER NOT NULL)")
FETCH_ROW = "SELECT V0, Vm, Rho, Kappa, Sigma FROM HestonParameters WHERE Name = ?"
INSERT_UPDATE = ("INSERT INTO HestonParameters VALUES(?, ?, ?, ?, ?, ?, strftime('%s','now')) ON CONFLICT(Name) "
                 "DO UPDATE SET V0 = excluded.V0, Vm = excluded.Vm, Rho = excluded.Rho, Kappa = excluded.Kappa, "
                 "Sigma = excluded.Sigma, ComputedAt = excluded.ComputedAt")


class NotFound(KeyError):
    """No row for the name (the reference throws DBException, DB.cpp:19)."""


class ParamsDB:
    def __init__(self, path: str | Path = "HParams.db"):
        self._db = sqlite3.connect(str(path))
        self._db.execute(CREATE_TABLE)
        self._db.commit()

    def fetch(self, name: str, r: float = 0.0, q: float = 0.0) -> Params:
        """Parameters of one underlying; r and q are not stored by the reference."""
        row = self._db.execute(FETCH_ROW, (name,)).fetchone()
        if row is None:
            raise NotFound(name)
        v0, vm, rho, kappa, sigma = row
        return Params(v0, vm, rho, kappa, sigma, r, q)

    def insertupdate(self, params: Params, name: str) -> None:
        self._db.execute(INSERT_UPDATE, (name, params.v0, params.theta, params.rho, params.kappa, params.sigma))
        self._db.commit()

    def names(self) -> list[str]:
        return [r[0] for r in self._db.execute("SELECT Name FROM HestonParameters ORDER BY Name")]

    def request(self, name: str, S0: float, options: Options, seed: int = 42, r: float = 0.0,
                q: float = 0.0, stream: int = 0) -> Request:
        return Request(self.fetch(name, r, q), S0, options, seed, stream)

    def close(self) -> None:
        self._db.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
