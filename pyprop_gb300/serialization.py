"""Saving and loading wavefunctions and tensor potentials (checkpoints).

The reference stores them in HDF5 through pytables (``pyprop/serialization/WavefunctionHDF.py``,
``TensorPotentialHDF.py``, ``CommonHDF.py``): one dataset per wavefunction, one group per tensor
potential with the data, the basis pairs and storage id of every rank, and the config as an
attribute. No HDF5 library is available here, so the same layout lives in a numpy ``.npz``
archive: dataset paths become keys (``/`` kept as the separator), attributes are keys with a
``#`` suffix. Several wavefunctions and potentials can share one file; saving a path replaces
it and keeps the others (the file is rewritten through a temporary file and renamed).

* ``SaveWavefunction(filename, datasetPath, psi, conf=None)`` / ``LoadWavefunction(filename,
  datasetPath, psi)`` (``SaveWavefunctionHDF`` / ``LoadWavefunctionHDF``, WavefunctionHDF.py:2-101):
  the complex128 data in the wavefunction's C order; loading checks the shape.
* ``SaveTensorPotential(filename, groupPath, potential, distributedModel=None, conf=None)`` /
  ``LoadTensorPotential(filename, groupPath, potential, distributedModel=None)``
  (TensorPotentialHDF.py:10-170): the potential data with ``basisPairs<i>`` and the storage id
  of each rank; loading refuses a file whose basis pairs differ from the potential's geometry
  (``CheckLocalSlab``, :140-157). A factorized two-electron term is stored as its factors
  (angular coefficients, weights, radial stencils). ``distributedModel`` is accepted for the
  reference's signature; the GPU path runs one process per wavefunction.
* ``Problem.SaveCheckpoint`` / ``LoadCheckpoint`` (in :mod:`pyprop_gb300.problem`) put the
  wavefunction and the propagated time in one file, so a long propagation can resume.
"""
from __future__ import annotations

import io
import os
import tempfile

import numpy as np


def _norm(path):
    path = "/" + str(path).strip("/")
    if path == "/":
        raise ValueError("a dataset path other than '/' is required")
    return path


def _read(filename):
    if not os.path.exists(filename):
        return {}
    with np.load(filename, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def _write(filename, entries):
    d = os.path.dirname(os.path.abspath(filename)) or "."
    fd, tmp = tempfile.mkstemp(dir=d, suffix=".npz")
    os.close(fd)
    try:
        with open(tmp, "wb") as fh:
            np.savez(fh, **entries)
        os.replace(tmp, filename)
    finally:
        if os.path.exists(tmp):
            os.remove(tmp)


def _drop(entries, path):
    for k in [k for k in entries if k == path or k.startswith(path + "/") or k.startswith(path + "#")]:
        del entries[k]


def _config_text(conf):
    if conf is None:
        return None
    cfg = getattr(conf, "cfgObj", None)
    if cfg is None:
        return str(conf)
    buf = io.StringIO()
    cfg.write(buf)
    return buf.getvalue()


def _host(psi):
    data = psi.GetData()
    if hasattr(data, "detach"):
        return data.detach().to("cpu").numpy()
    return np.asarray(data)


def SaveWavefunction(filename, datasetPath, psi, conf=None):
    """Store psi's data (complex128, C order) at ``datasetPath``; ``conf`` (a Config) is kept
    as the dataset's configObject attribute."""
    path = _norm(datasetPath)
    entries = _read(filename)
    _drop(entries, path)
    entries[path] = np.ascontiguousarray(_host(psi), dtype=np.complex128)
    text = _config_text(conf)
    if text is not None:
        entries[path + "#configObject"] = np.array(text)
    _write(filename, entries)


def LoadWavefunction(filename, datasetPath, psi):
    """Copy the dataset into psi (its shape must equal the wavefunction's)."""
    path = _norm(datasetPath)
    with np.load(filename, allow_pickle=False) as z:
        if path not in z.files:
            raise KeyError("no dataset %s in %s" % (path, filename))
        data = z[path]
    shape = tuple(psi.GetRepresentation().GetFullShape())
    if tuple(data.shape) != shape:
        raise ValueError("dataset %s has shape %s, the wavefunction %s" % (path, data.shape, shape))
    psi.SetData(data)
    return psi


def GetConfigText(filename, datasetPath):
    """The config stored with a dataset, as INI text (None if there is none)."""
    path = _norm(datasetPath)
    with np.load(filename, allow_pickle=False) as z:
        key = path + "#configObject"
        return str(z[key]) if key in z.files else None


def SaveTensorPotential(filename, groupPath, potential, distributedModel=None, conf=None):
    """Store a TensorPotential under ``groupPath``: ``potential`` (reference-layout data) or the
    factors of a factorized term, plus ``basisPairs<i>`` and ``storageId<i>`` of each rank."""
    path = _norm(groupPath)
    entries = _read(filename)
    _drop(entries, path)
    for i, geom in enumerate(potential.GeometryList):
        pairs = geom.GetBasisPairs()
        entries["%s/basisPairs%d" % (path, i)] = np.zeros((0, 2), np.int32) if pairs is None else np.asarray(pairs)
        entries["%s/basisPairs%d#storageId" % (path, i)] = np.array(geom.GetStorageId())
    fac = getattr(potential, "Factors", None)
    if fac is not None:
        entries[path + "/factors/coefs"] = fac.coefs
        entries[path + "/factors/weights"] = fac.weights
        entries[path + "/factors/stencil"] = fac.stencil
        entries[path + "/factors/pairs"] = np.zeros((0, 2), np.int32) if fac.pairs is None else fac.pairs
        entries[path + "/factors#kb"] = np.array(fac.kb)
        entries[path + "/factors#nangular"] = np.array(fac.nangular)
    else:
        entries[path + "/potential"] = np.ascontiguousarray(potential.PotentialData)
    text = _config_text(conf)
    if text is not None:
        entries[path + "#configObject"] = np.array(text)
    _write(filename, entries)


def CheckBasisPairs(filename, groupPath, geometryList):
    """True when the stored basis pairs of every rank equal those of ``geometryList``."""
    path = _norm(groupPath)
    with np.load(filename, allow_pickle=False) as z:
        for i, geom in enumerate(geometryList):
            key = "%s/basisPairs%d" % (path, i)
            if key not in z.files:
                return False
            pairs = geom.GetBasisPairs()
            new = np.zeros((0, 2), np.int32) if pairs is None else np.asarray(pairs)
            old = z[key]
            if old.shape != new.shape or not np.all(old == new):
                return False
            if str(z[key + "#storageId"]) != geom.GetStorageId():
                return False
    return True


def LoadTensorPotential(filename, groupPath, potential, distributedModel=None):
    """Fill ``potential`` (whose GeometryList is set up) from the file, after checking that the
    stored basis pairs match its geometry."""
    from .tensorpotential import FactoredPotential
    path = _norm(groupPath)
    if not CheckBasisPairs(filename, path, potential.GeometryList):
        raise ValueError("basis pairs in %s:%s differ from the potential's geometry" % (filename, path))
    with np.load(filename, allow_pickle=False) as z:
        if path + "/potential" in z.files:
            potential.Factors = None
            potential.PotentialData = z[path + "/potential"]
            return potential
        pairs = z[path + "/factors/pairs"]
        geoms = potential.GeometryList
        radial_pairs = (geoms[1].GetBasisPairs(), geoms[2].GetBasisPairs())
        potential.Factors = FactoredPotential(pairs if len(pairs) else None, z[path + "/factors/coefs"],
                                              z[path + "/factors/weights"], z[path + "/factors/stencil"],
                                              radial_pairs, int(z[path + "/factors#kb"]),
                                              int(z[path + "/factors#nangular"]))
        potential.PotentialData = None
    return potential
