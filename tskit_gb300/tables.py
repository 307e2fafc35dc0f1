"""Columnar tree-sequence tables on the host (numpy), the input to the device path.

Only the columns the statistics path reads are kept: node time and flags,
edges, site positions and ancestral states, and mutations with their derived
states.  The two edge indexes and the per-mutation integer allele codes are
derived here once per tree sequence; everything downstream runs on the GPU.

Semantics follow the reference:
  * edge sort order (time[parent], parent, child, left) -- c/tskit/tables.c
    (tsk_table_collection_sort / check_integrity with TSK_CHECK_EDGE_ORDERING);
  * insertion index sorted by (left, time[parent], parent, child) and removal
    index by (right, -time[parent], -parent, -child) -- c/tskit/tables.c:11393-11450;
  * allele numbering per site: the ancestral state is allele 0 and each new
    derived-state string gets the next number in mutation order, the
    "alternate" allele of a mutation is its parent mutation's derived state or
    the ancestral state -- c/tskit/trees.c:1525-1612 (get_allele_weights).
"""
from __future__ import annotations

import dataclasses

import numpy as np

NODE_IS_SAMPLE = 1
NULL = -1


def _ragged(strings, default=b""):
    data = []
    offsets = [0]
    for s in strings:
        if isinstance(s, str):
            s = s.encode()
        data.append(s)
        offsets.append(offsets[-1] + len(s))
    return (
        np.frombuffer(b"".join(data), dtype=np.uint8).copy(),
        np.array(offsets, dtype=np.uint64),
    )


@dataclasses.dataclass
class Tables:
    sequence_length: float
    node_time: np.ndarray
    node_flags: np.ndarray
    edge_left: np.ndarray
    edge_right: np.ndarray
    edge_parent: np.ndarray
    edge_child: np.ndarray
    site_position: np.ndarray
    site_ancestral_state: np.ndarray
    site_ancestral_state_offset: np.ndarray
    mutation_site: np.ndarray
    mutation_node: np.ndarray
    mutation_parent: np.ndarray
    mutation_derived_state: np.ndarray
    mutation_derived_state_offset: np.ndarray
    edge_insertion_order: np.ndarray | None = None
    edge_removal_order: np.ndarray | None = None
    time_uncalibrated: bool = False
    # the node table's individual column and the number of individuals
    # (read from .trees files; pca over individuals groups nodes by it)
    node_individual: np.ndarray | None = None
    num_individuals: int = 0

    # ------------------------------------------------------------ building
    @classmethod
    def from_columns(
        cls,
        sequence_length,
        node_time,
        node_flags,
        edge_left,
        edge_right,
        edge_parent,
        edge_child,
        site_position=(),
        site_ancestral_state=None,
        mutation_site=(),
        mutation_node=(),
        mutation_parent=None,
        mutation_derived_state=None,
        sort=True,
    ):
        site_position = np.asarray(site_position, dtype=np.float64)
        S = len(site_position)
        if site_ancestral_state is None:
            site_ancestral_state = [b"0"] * S
        if isinstance(site_ancestral_state, tuple) and len(site_ancestral_state) == 2:
            anc, anc_off = site_ancestral_state
        else:
            anc, anc_off = _ragged(site_ancestral_state)
        mutation_site = np.asarray(mutation_site, dtype=np.int32)
        M = len(mutation_site)
        if mutation_parent is None:
            mutation_parent = np.full(M, NULL, dtype=np.int32)
        if mutation_derived_state is None:
            mutation_derived_state = [b"1"] * M
        if isinstance(mutation_derived_state, tuple) and len(mutation_derived_state) == 2:
            der, der_off = mutation_derived_state
        else:
            der, der_off = _ragged(mutation_derived_state)
        t = cls(
            sequence_length=float(sequence_length),
            node_time=np.ascontiguousarray(node_time, dtype=np.float64),
            node_flags=np.ascontiguousarray(node_flags, dtype=np.uint32),
            edge_left=np.ascontiguousarray(edge_left, dtype=np.float64),
            edge_right=np.ascontiguousarray(edge_right, dtype=np.float64),
            edge_parent=np.ascontiguousarray(edge_parent, dtype=np.int32),
            edge_child=np.ascontiguousarray(edge_child, dtype=np.int32),
            site_position=site_position,
            site_ancestral_state=np.asarray(anc, dtype=np.uint8),
            site_ancestral_state_offset=np.asarray(anc_off, dtype=np.uint64),
            mutation_site=mutation_site,
            mutation_node=np.ascontiguousarray(mutation_node, dtype=np.int32),
            mutation_parent=np.ascontiguousarray(mutation_parent, dtype=np.int32),
            mutation_derived_state=np.asarray(der, dtype=np.uint8),
            mutation_derived_state_offset=np.asarray(der_off, dtype=np.uint64),
        )
        if sort:
            t.sort_edges()
        t.build_index()
        return t

    @classmethod
    def load(cls, path):
        """Read the statistics' columns of a ``.trees`` file (tskit's kastore
        container; the reader is ``tsg_kastore_*`` in the native library).
        The checks follow tsk_table_collection_load (c/tskit/tables.c:
        11580-11830): the format name and major version, the sequence
        length, required columns, column types, and ragged columns with
        their offsets (32- or 64-bit)."""
        import ctypes

        from . import _native as nat

        lib = nat.load()
        handle = ctypes.c_void_p()
        nat.check(lib.tsg_kastore_open(str(path).encode(), ctypes.byref(handle)))
        dtypes = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64,
                  np.uint64, np.float32, np.float64]
        try:
            def get(key, types, required=True):
                t = ctypes.c_int32()
                n = ctypes.c_int64()
                ptr = ctypes.c_void_p()
                code = lib.tsg_kastore_get(handle, key.encode(), ctypes.byref(t),
                                           ctypes.byref(n), ctypes.byref(ptr))
                if code != 0:
                    if required:
                        raise nat.LibraryError(code)
                    return None
                dt = np.dtype(dtypes[t.value])
                if dt not in [np.dtype(x) for x in types]:
                    raise nat.LibraryError(nat.ERR_BAD_COLUMN_TYPE)
                if n.value == 0:
                    return np.zeros(0, dtype=dt)
                buf = (ctypes.c_char * (n.value * dt.itemsize)).from_address(ptr.value)
                return np.frombuffer(buf, dtype=dt).copy()

            def ragged(key, nrows):
                data = get(key, [np.int8, np.uint8], required=False)
                off = get(key + "_offset", [np.uint32, np.uint64], required=False)
                if (data is None) != (off is None):
                    raise nat.LibraryError(nat.ERR_BOTH_COLUMNS_REQUIRED)
                if data is None:
                    raise nat.LibraryError(nat.ERR_REQUIRED_COL_NOT_FOUND)
                off = off.astype(np.uint64)
                if len(off) != nrows + 1 or off[0] != 0 or np.any(np.diff(off.astype(np.int64)) < 0) \
                        or off[-1] != len(data):
                    raise nat.LibraryError(nat.ERR_BAD_OFFSET)
                return data.view(np.uint8), off

            name = get("format/name", [np.int8])
            if name.tobytes() != b"tskit.trees":
                raise nat.LibraryError(nat.ERR_FILE_FORMAT)
            version = get("format/version", [np.uint32])
            if len(version) != 2:
                raise nat.LibraryError(nat.ERR_FILE_FORMAT)
            if version[0] < 12:
                raise nat.LibraryError(nat.ERR_FILE_VERSION_TOO_OLD)
            if version[0] > 12:
                raise nat.LibraryError(nat.ERR_FILE_VERSION_TOO_NEW)
            L = get("sequence_length", [np.float64])
            if len(L) != 1:
                raise nat.LibraryError(nat.ERR_FILE_FORMAT)
            time_units = get("time_units", [np.int8], required=False)

            def cols(keys, types):
                arrays = [get(k, t) for k, t in zip(keys, types)]
                if len({len(a) for a in arrays}) > 1:
                    raise nat.LibraryError(nat.ERR_FILE_FORMAT)
                return arrays

            node_time, node_flags = cols(["nodes/time", "nodes/flags"], [[np.float64], [np.uint32]])
            node_individual = get("nodes/individual", [np.int32], required=False)
            individual_flags = get("individuals/flags", [np.uint32], required=False)
            left, right, parent, child = cols(
                ["edges/left", "edges/right", "edges/parent", "edges/child"],
                [[np.float64], [np.float64], [np.int32], [np.int32]])
            (position,) = cols(["sites/position"], [[np.float64]])
            anc, anc_off = ragged("sites/ancestral_state", len(position))
            msite, mnode, mparent = cols(["mutations/site", "mutations/node", "mutations/parent"],
                                         [[np.int32]] * 3)
            der, der_off = ragged("mutations/derived_state", len(msite))
        finally:
            lib.tsg_kastore_free(handle)
        t = cls.from_columns(float(L[0]), node_time, node_flags, left, right, parent, child,
                             site_position=position, site_ancestral_state=(anc, anc_off),
                             mutation_site=msite, mutation_node=mnode, mutation_parent=mparent,
                             mutation_derived_state=(der, der_off))
        if time_units is not None and time_units.tobytes() == b"uncalibrated":
            t.time_uncalibrated = True
        if node_individual is not None and len(node_individual) == len(node_time):
            t.node_individual = node_individual
            t.num_individuals = 0 if individual_flags is None else len(individual_flags)
        return t

    @property
    def num_nodes(self):
        return len(self.node_time)

    @property
    def num_edges(self):
        return len(self.edge_left)

    @property
    def num_sites(self):
        return len(self.site_position)

    @property
    def num_mutations(self):
        return len(self.mutation_site)

    def samples(self):
        return np.flatnonzero(self.node_flags & NODE_IS_SAMPLE).astype(np.int32)

    def sort_edges(self):
        """Sort edges by (time[parent], parent, child, left)."""
        tp = self.node_time[self.edge_parent]
        order = np.lexsort((self.edge_left, self.edge_child, self.edge_parent, tp))
        for name in ("edge_left", "edge_right", "edge_parent", "edge_child"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name)[order]))

    def build_index(self):
        tp = self.node_time[self.edge_parent]
        self.edge_insertion_order = np.lexsort(
            (self.edge_child, self.edge_parent, tp, self.edge_left)
        ).astype(np.int32)
        self.edge_removal_order = np.lexsort(
            (-self.edge_child, -self.edge_parent, -tp, self.edge_right)
        ).astype(np.int32)

    def decapitated_topology(self, time):
        """The nodes and edges of ``decapitate(time)`` (python/tskit/trees.py:
        7396-7437: split_edges, then delete_older): edges whose child is at
        least as old as ``time`` are removed, and every edge spanning
        ``time`` gets its own new parent node at ``time`` (not a sample).
        Sites and mutations are left out: this is the input of branch
        statistics restricted to the material younger than ``time``."""
        tp = self.node_time[self.edge_parent]
        tc = self.node_time[self.edge_child]
        keep = tp <= time
        split = (tc < time) & (tp > time)
        N = self.num_nodes
        ns = int(np.count_nonzero(split))
        parent = self.edge_parent.copy()
        parent[split] = N + np.arange(ns, dtype=np.int32)
        sel = keep | split
        node_individual = None
        if self.node_individual is not None:
            node_individual = np.concatenate(
                [self.node_individual, np.full(ns, NULL, dtype=np.int32)])
        t = Tables.from_columns(
            self.sequence_length,
            np.concatenate([self.node_time, np.full(ns, float(time))]),
            np.concatenate([self.node_flags, np.zeros(ns, dtype=np.uint32)]),
            self.edge_left[sel], self.edge_right[sel], parent[sel], self.edge_child[sel])
        t.time_uncalibrated = self.time_uncalibrated
        t.node_individual = node_individual
        t.num_individuals = self.num_individuals
        return t

    # ------------------------------------------------------------ checks
    def check(self):
        """Raise ValueError unless the tables form a valid sorted tree sequence
        for the statistics path (the subset of tsk_table_collection_check_integrity
        the sweep relies on)."""
        N = self.num_nodes
        L = self.sequence_length
        if not (L > 0):
            raise ValueError("sequence_length must be positive")
        e_p, e_c = self.edge_parent, self.edge_child
        if self.num_edges:
            if e_p.min() < 0 or e_p.max() >= N or e_c.min() < 0 or e_c.max() >= N:
                raise ValueError("edge node out of bounds")
            if np.any(self.edge_left < 0) or np.any(self.edge_right > L):
                raise ValueError("edge interval out of bounds")
            if np.any(self.edge_left >= self.edge_right):
                raise ValueError("bad edge interval")
            if np.any(self.node_time[e_p] <= self.node_time[e_c]):
                raise ValueError("bad node time ordering")
        if self.num_sites:
            if np.any(np.diff(self.site_position) <= 0):
                raise ValueError("sites must be sorted by strictly increasing position")
            if self.site_position[0] < 0 or self.site_position[-1] >= L:
                raise ValueError("site position out of bounds")
        if self.num_mutations:
            if np.any(np.diff(self.mutation_site) < 0):
                raise ValueError("mutations must be sorted by site")
            if self.mutation_site.min() < 0 or self.mutation_site.max() >= self.num_sites:
                raise ValueError("mutation site out of bounds")
            if self.mutation_node.min() < 0 or self.mutation_node.max() >= N:
                raise ValueError("mutation node out of bounds")

    # ------------------------------------------------------------ alleles
    def allele_codes(self):
        """Per-mutation (allele, alternate allele) integer codes.

        Returns (allele, parent_allele, num_alleles_per_site) as int32 arrays.
        The numbering restates get_allele_weights (c/tskit/trees.c:1525-1612)
        so that string comparisons never reach the device.
        """
        M = self.num_mutations
        allele = np.zeros(M, dtype=np.int32)
        alt = np.zeros(M, dtype=np.int32)
        nalleles = np.ones(self.num_sites, dtype=np.int32)
        if M == 0:
            return allele, alt, nalleles
        anc = self.site_ancestral_state.tobytes()
        anc_off = self.site_ancestral_state_offset
        der = self.mutation_derived_state.tobytes()
        der_off = self.mutation_derived_state_offset
        ms = self.mutation_site
        mp = self.mutation_parent
        # fast path: every derived state differs from its site's ancestral
        # state, every site has one mutation and no mutation has a parent
        starts = np.searchsorted(ms, np.arange(self.num_sites + 1))
        counts = np.diff(starts)
        if np.all(counts <= 1) and np.all(mp == NULL):
            dl = np.diff(der_off.astype(np.int64))
            same = np.zeros(M, dtype=bool)
            for j in np.flatnonzero(dl == np.diff(anc_off.astype(np.int64))[ms]):
                s = ms[j]
                same[j] = der[der_off[j]:der_off[j + 1]] == anc[anc_off[s]:anc_off[s + 1]]
            allele[:] = np.where(same, 0, 1)
            nalleles[ms[~same]] = 2
            return allele, alt, nalleles
        for s in range(self.num_sites):
            a, b = starts[s], starts[s + 1]
            if a == b:
                continue
            table = [anc[anc_off[s]:anc_off[s + 1]]]
            for j in range(a, b):
                d = der[der_off[j]:der_off[j + 1]]
                try:
                    k = table.index(d)
                except ValueError:
                    k = len(table)
                    table.append(d)
                allele[j] = k
                if mp[j] == NULL:
                    alt[j] = 0
                else:
                    pd = der[der_off[mp[j]]:der_off[mp[j] + 1]]
                    alt[j] = table.index(pd)
            nalleles[s] = len(table)
        return allele, alt, nalleles

    # ------------------------------------------------------------ interop
    def to_dict(self):
        return {f.name: getattr(self, f.name) for f in dataclasses.fields(self)}

    @classmethod
    def from_npz(cls, data, prefix=""):
        kw = {}
        for f in dataclasses.fields(cls):
            key = prefix + f.name
            if key in data:
                v = data[key]
                if f.name == "sequence_length":
                    v = float(v)
                elif f.name == "time_uncalibrated":
                    v = bool(v)
                elif f.name == "num_individuals":
                    v = int(v)
                kw[f.name] = v
        t = cls(**kw)
        if t.edge_insertion_order is None:
            t.build_index()
        return t

    def save_npz_dict(self, prefix=""):
        return {prefix + k: np.asarray(v) for k, v in self.to_dict().items() if v is not None}
