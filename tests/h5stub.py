"""An in-memory stand-in for the few ``h5py`` calls the result store makes.

h5py is installed on neither test machine. This module records what a
writer puts into a file -- groups, datasets (a copy of the data and the
creation keywords) and attributes -- and lets a reader open it again:
``File(path, "w")`` writes a unique token to ``path`` on disk (so atomic
renames move a real file) and keeps the tree under that token;
``File(path, "r")`` reads the token back. ``install(monkeypatch)`` puts the
module in ``sys.modules["h5py"]`` for one test.
"""

from __future__ import annotations

import sys
import types
import uuid
from pathlib import Path

import numpy as np

TREES: dict[str, "Group"] = {}


class Attrs(dict):
    pass


class Dataset:
    def __init__(self, data, kwargs):
        self.data = np.array(data, copy=True)
        self.kwargs = dict(kwargs)
        self.attrs = Attrs()

    @property
    def shape(self):
        return self.data.shape

    @property
    def dtype(self):
        return self.data.dtype

    def __getitem__(self, key):
        return self.data[key]


class Group:
    def __init__(self):
        self.attrs = Attrs()
        self.children: dict[str, object] = {}

    def _walk(self, path: str):
        node = self
        for part in [p for p in path.split("/") if p]:
            node = node.children[part]
        return node

    def create_group(self, name: str) -> "Group":
        g = Group()
        self.children[name] = g
        return g

    def create_dataset(self, name: str, data=None, **kwargs) -> Dataset:
        d = Dataset(data, kwargs)
        self.children[name] = d
        return d

    def __getitem__(self, path: str):
        return self._walk(path)

    def __contains__(self, path: str) -> bool:
        try:
            self._walk(path)
            return True
        except KeyError:
            return False


class File(Group):
    def __init__(self, path, mode: str = "r"):
        super().__init__()
        self.path = Path(path)
        if mode == "w":
            token = uuid.uuid4().hex
            self.path.write_text(token)
            TREES[token] = self
        else:
            if not self.path.exists():
                raise OSError(f"no such file: {self.path}")
            tree = TREES[self.path.read_text()]
            self.attrs, self.children = tree.attrs, tree.children

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def close(self):
        pass


def module() -> types.ModuleType:
    m = types.ModuleType("h5py")
    m.File, m.Group, m.Dataset = File, Group, Dataset
    return m


def install(monkeypatch) -> types.ModuleType:
    m = module()
    monkeypatch.setitem(sys.modules, "h5py", m)
    return m


def tree(path) -> File:
    """The recorded tree of a file written through the stub."""
    return File(path, "r")
