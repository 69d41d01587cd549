"""Measurement bins and their files in the reference's on-disk layout.

The reference's MeasurementSystem (src/mod_meas.f90) keeps
data(total_width, nmeas, nbins): one vector per finished measurement, laid
out by the observable namelist (:587-627: every ``&observable`` group in
file order, a field followed by its ``_k`` transform, offsets assigned by
ms_finalize_layout :697-716).  ms_begin_measure (:729-763) fills
measurement cur_meas of bin cur_bin; a full bin is averaged (the real part,
ms_compute_one_bin_mean :853-866) and appended to the stream file
``temp/tempout_core[<id>].bin`` with a line in ``temp/tempout_core_count.dat``
(:883-944); ms_data_analyse (:845-852, :946-973) writes all bin means,
mean(total_width, nbins) column-major, to ``data/out_core[<id>].bin``;
ms_output_reading_guide (:975-1017) describes the layout in
``data/reading_guide.nml``.  The post-processing scripts of the reference
read exactly these files.

The device measurement writes records in a fixed order (the three
scalars, then each field with its k-space transform; model.SCALAR_NAMES,
model.FIELD_NAMES); ``MeasurementBins`` places every record into the
namelist layout by name, leaving observables the device does not measure
at zero as the reference does for names it has no handle for.
"""
from __future__ import annotations

import os

import numpy as np

from .model import FIELD_NAMES, SCALAR_NAMES, Model

KIND_SCALAR, KIND_FIELD = 1, 2      # mod_meas.f90:7


def device_slots(m: Model) -> dict[str, tuple[int, int]]:
    """name -> (offset, width) in a device measurement record."""
    nc = m.lat.n_cell
    ns, nf = len(SCALAR_NAMES), len(FIELD_NAMES)
    out = {n: (i, 1) for i, n in enumerate(SCALAR_NAMES)}
    # r-space block of every field, then the k-space block (meas.cu
    # k_meas_finish writes field f's transform at ns + (nf + f) * nc)
    for f, n in enumerate(FIELD_NAMES):
        out[n] = (ns + f * nc, nc)
        out[n + "_k"] = (ns + (nf + f) * nc, nc)
    return out


def reference_layout(m: Model, observables=None) -> list[dict]:
    """The observable list of ms_init_from_namelist / ms_finalize_layout:
    [{name, kind, width, offset_lo, offset_hi}] with 1-based offsets."""
    obs = list(observables if observables is not None else m.spec.observables)
    if not obs:
        raise ValueError("no observable groups (ms_init_from_namelist needs at least one)")
    fw = int(np.prod(m.lat.dlength))
    entries = []
    for name, kind in obs:
        k = str(kind).strip().lower()
        if k in ("scalar", "s", "sc", "1"):
            entries.append((name.strip(), KIND_SCALAR, 1))
        elif k in ("field", "f", "array", "a"):
            entries.append((name.strip(), KIND_FIELD, fw))
            entries.append((name.strip() + "_k", KIND_FIELD, fw))
        else:
            raise ValueError(f"unknown observable kind {kind!r} (name={name})")
    names = [e[0] for e in entries]
    if len(set(names)) != len(names):
        raise ValueError("duplicate observable name")
    out, cursor = [], 1
    for name, kind, width in entries:
        out.append({"name": name, "kind": kind, "width": width, "offset_lo": cursor,
                    "offset_hi": cursor + width - 1})
        cursor += width
    return out


def _fortran_ld(key: str, v) -> str:
    """One `write(lun,*) 'key=', value` line as gfortran's list-directed
    output writes it."""
    if isinstance(v, str):
        return f" {key}=\"{v}\""
    return f" {key}={int(v):12d}"


class MeasurementBins:
    """data(total_width, nmeas, nbins) with the reference's bin cadence and
    output files.  core_id None writes the non-MPI file names, an integer
    the MPI ones (tempout_core<id>.bin, out_core<id>.bin)."""

    def __init__(self, m: Model, *, nbins: int | None = None, nmeas: int | None = None,
                 output_addr: str = "data/", core_id: int | None = None, observables=None,
                 output_format: str = "f18.8", reading_guide: str = "reading_guide.nml", write: bool = True):
        self.m = m
        self.nbins = int(nbins if nbins is not None else m.spec.nbin_per_core)
        self.nmeas = int(nmeas if nmeas is not None else m.spec.nmeas_per_bin)
        if self.nbins <= 0 or self.nmeas <= 0:
            raise ValueError("nbins/nmeas must be > 0")
        self.layout = reference_layout(m, observables)
        self.total_width = self.layout[-1]["offset_hi"]
        self.field_width = int(np.prod(m.lat.dlength))
        self.data = np.zeros((self.total_width, self.nmeas, self.nbins), dtype=np.complex128, order="F")
        self.mean = np.zeros((self.total_width, self.nbins), order="F")
        self.cur_bin, self.cur_meas = 1, 1
        self.addr, self.core_id, self.write = output_addr, core_id, write
        self.output_format, self.reading_guide = output_format, reading_guide
        slots = device_slots(m)
        # (reference range, device range) for every observable the device measures
        self._map = [(e["offset_lo"] - 1, slots[e["name"]][0], e["width"]) for e in self.layout
                     if e["name"] in slots and slots[e["name"]][1] == e["width"]]
        if write:
            os.makedirs(os.path.join(output_addr, "data"), exist_ok=True)
            os.makedirs(os.path.join(output_addr, "temp"), exist_ok=True)
            self.write_reading_guide()

    # ---- files -----------------------------------------------------------
    def _core(self, stem: str) -> str:
        return f"{stem}{'' if self.core_id is None else self.core_id}.bin"

    @property
    def out_file(self) -> str:
        return os.path.join(self.addr, "data", self._core("out_core"))

    @property
    def temp_file(self) -> str:
        return os.path.join(self.addr, "temp", self._core("tempout_core"))

    def write_reading_guide(self, n_cores: int | None = None, mpi_nblock: int | None = None,
                            mpi_one_block: int | None = None):
        """ms_output_reading_guide (mod_meas.f90:975-1017)."""
        lines = [" &basics", _fortran_ld("n_obs", len(self.layout)), _fortran_ld("total_width", self.total_width),
                 _fortran_ld("n_bins", self.nbins), _fortran_ld("n_meas_per_bin", self.nmeas),
                 _fortran_ld("field_width", self.field_width), _fortran_ld("size_of_dp", 8)]
        if n_cores is not None:
            lines += [_fortran_ld("n_cores", n_cores), _fortran_ld("MPI_nblock", mpi_nblock or 1),
                      _fortran_ld("MPI_one_block", mpi_one_block or n_cores)]
        lines += [_fortran_ld("output_format", self.output_format), " /", " "]
        for e in self.layout:
            lines += [" &obs", _fortran_ld("name", e["name"]), _fortran_ld("kind", e["kind"]),
                      _fortran_ld("width", e["width"]), _fortran_ld("offset_lo", e["offset_lo"]),
                      _fortran_ld("offset_hi", e["offset_hi"]), " /", " "]
        with open(os.path.join(self.addr, "data", self.reading_guide), "w") as f:
            f.write("\n".join(lines) + "\n")

    # ---- records ----------------------------------------------------------
    def to_layout(self, record: np.ndarray) -> np.ndarray:
        """A device record (complex, model.record_width) in the namelist layout."""
        v = np.zeros(self.total_width, dtype=np.complex128)
        for lo, dlo, w in self._map:
            v[lo:lo + w] = record[dlo:dlo + w]
        return v

    def add(self, record: np.ndarray):
        """One finished measurement (the window average of ms_begin_measure)."""
        if self.cur_bin > self.nbins:
            raise RuntimeError("begin_measure: no more bins left")
        self.data[:, self.cur_meas - 1, self.cur_bin - 1] = self.to_layout(np.asarray(record))
        self.cur_meas += 1
        if self.cur_meas > self.nmeas:
            b = self.cur_bin
            self.mean[:, b - 1] = np.real(self.data[:, :, b - 1]).sum(axis=1) / float(self.nmeas)
            if self.write:
                self._append_bin(b)
            self.cur_meas = 1
            self.cur_bin += 1

    def add_records(self, records):
        for r in np.atleast_2d(records):
            self.add(r)

    def _append_bin(self, b: int):
        """ms_output_bin_data + ms_output_bin_count (mod_meas.f90:883-944)."""
        with open(self.temp_file, "ab") as f:
            f.write(np.ascontiguousarray(self.mean[:, b - 1], dtype="<f8").tobytes())
        with open(os.path.join(self.addr, "temp", "tempout_core_count.dat"), "a") as f:
            f.write(f"C{(self.core_id or 0):4d}   |    B{b:4d}\n")

    def finish(self) -> np.ndarray:
        """ms_data_analyse: every bin's mean, written to out_core(.bin) as
        mean(total_width, nbins) in column-major doubles."""
        for b in range(self.nbins):
            self.mean[:, b] = np.real(self.data[:, :, b]).sum(axis=1) / float(self.nmeas)
        if self.write:
            with open(self.out_file, "wb") as f:
                f.write(np.asfortranarray(self.mean, dtype="<f8").tobytes(order="F"))
        return self.mean

    def estimate(self) -> tuple[np.ndarray, np.ndarray]:
        """Mean over the bins and its standard error (bins as independent
        samples), per entry of the layout."""
        n = self.nbins
        mu = self.mean.mean(axis=1)
        err = np.sqrt(((self.mean - mu[:, None]) ** 2).sum(axis=1) / (n * (n - 1))) if n > 1 else np.zeros_like(mu)
        return mu, err

    def observable(self, name: str) -> np.ndarray:
        """The (width, nbins) bin means of one observable."""
        for e in self.layout:
            if e["name"] == name:
                return self.mean[e["offset_lo"] - 1:e["offset_hi"]]
        raise KeyError(name)


def read_out_core(path: str, total_width: int, nbins: int) -> np.ndarray:
    """out_core(.bin) back as (total_width, nbins), as the post-processing
    reads it."""
    return np.fromfile(path, dtype="<f8").reshape((total_width, nbins), order="F")
