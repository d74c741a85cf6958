"""Reader of the ROOT file format, limited to what the multifit data files use.

The reference reads its inputs through ROOT itself: `TFile`, `TTree::
SetBranchAddress` / `GetEntry` on the `Samples` tree (io/src/ecal_data_io.cpp:
6-24, multifit_cpu/src/multifit.cpp:86-92) and the pulse-shape `TGraph` plus the
`Tail` tree of `EmptyFile.root` (multifit_cpu/interface/Pulse.h:79-98). ROOT is
not a dependency of this engine, so this module reads those records from the
documented on-disk layout, with the standard library's zlib and lzma:

- file header: ``"root"``, version (>= 1000000: 64-bit seeks), fBEGIN, fEND,
  fSeekFree, fNbytesFree, nfree, fNbytesName, fUnits, fCompress, ...;
- a key (TKey) in front of every record: Nbytes, version (> 1000: 64-bit
  seeks), ObjLen, Datime, KeyLen, Cycle, SeekKey, SeekPdir, then the class
  name, name and title as ROOT strings (1 length byte, or 255 and an int32);
- a directory record: version, two dates, NbytesKeys, NbytesName, SeekDir,
  SeekParent, SeekKeys; the keys list at SeekKeys is a key, an int32 count and
  that many key headers;
- a compressed record: blocks of a 9-byte header (2-letter algorithm, method
  byte, 3-byte little-endian compressed and uncompressed sizes) and data;
- a basket (TBasket) key adds version, BufferSize, NevBufSize, NevBuf, Last
  and a flag byte to the key; its buffer holds the entries up to Last, then,
  for entries of varying size, an int32 count and the entries' start offsets
  (relative to the key start);
- a streamed object starts with a byte count (bit 30 set) and a version; base
  classes (TNamed, TAttLine, TAttFill, TAttMarker) are skipped by their byte
  counts; `TTree` continues with fEntries (int64), `TGraph` with fNpoints and
  the fX and fY arrays (a presence byte, then fNpoints big-endian doubles).

All numbers are big-endian. A branch's entries are gathered from its basket
keys in file order (the order ROOT writes them while the tree fills) and
checked against the tree's fEntries, so a file whose baskets stayed inside the
tree record, or two trees of one name, raise instead of returning a partial
column. LZ4 and ZSTD blocks and ROOT's pre-zlib compression are not
supported and raise. Nothing here runs on the GPU.
"""
from __future__ import annotations

import functools
import lzma
import os
import struct
import zlib
from dataclasses import dataclass

import numpy as np

BYTECOUNT_FLAG = 0x40000000
IS_SORTED_X = 1 << 14  # TGraph::kIsSortedX in TObject::fBits


class RootFormatError(ValueError):
    """The file is not a ROOT file this reader can decode, or it is damaged."""


def _checked(fn):
    """Reports a damaged record as RootFormatError, whatever low-level error
    (short buffer, bad index, corrupt compressed block) decoding it hit."""

    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        try:
            return fn(*args, **kwargs)
        except (RootFormatError, KeyError):
            raise
        except (struct.error, IndexError, ValueError, zlib.error, lzma.LZMAError) as e:
            raise RootFormatError(f"malformed record ({type(e).__name__}: {e})") from e

    return wrapper


@dataclass
class Key:
    """One TKey header: where a record lies and what it holds."""

    pos: int
    nbytes: int
    version: int
    objlen: int
    keylen: int
    cycle: int
    seek_key: int
    seek_pdir: int
    class_name: str
    name: str
    title: str
    header_end: int  # file offset just after the title

    @property
    def compressed(self) -> bool:
        return self.objlen > self.nbytes - self.keylen


@dataclass
class Basket:
    key: Key
    nev_buf: int
    nev_buf_size: int
    last: int  # end of the entry data, relative to the key start


def _tstring(buf, p: int):
    n = buf[p]
    p += 1
    if n == 255:
        (n,) = struct.unpack_from(">i", buf, p)
        p += 4
    return bytes(buf[p:p + n]).decode("latin-1"), p + n


def _skip_streamed(buf, p: int, what: str) -> int:
    """Skips one streamed object (byte count + content) starting at p."""
    (bc,) = struct.unpack_from(">I", buf, p)
    if not bc & BYTECOUNT_FLAG:
        raise RootFormatError(f"{what}: no byte count at offset {p}")
    end = p + 4 + (bc & ~BYTECOUNT_FLAG)
    if end > len(buf):
        raise RootFormatError(f"{what}: byte count runs past the record")
    return end


def _skip_named_and_attributes(buf, what: str):
    """Positions after the class header, TNamed, TAttLine, TAttFill and
    TAttMarker of a TTree or TGraph record; also returns TObject::fBits."""
    p = 6  # byte count and version of the class itself
    # TNamed: byte count, version, then TObject: version, fUniqueID, fBits
    (bits,) = struct.unpack_from(">I", buf, p + 6 + 2 + 4)
    for base in ("TNamed", "TAttLine", "TAttFill", "TAttMarker"):
        p = _skip_streamed(buf, p, f"{what} {base}")
    return p, bits


class RootFile:
    """Read-only view of a ROOT file, read whole into memory (the multifit
    data files are a few MB)."""

    @_checked
    def __init__(self, source):
        if isinstance(source, (bytes, bytearray, memoryview)):
            self.path = "<bytes>"
            self.data = bytes(source)
        else:
            self.path = os.fspath(source)
            with open(self.path, "rb") as f:
                self.data = f.read()
        d = self.data
        if len(d) < 64 or d[:4] != b"root":
            raise RootFormatError(f"{self.path}: not a ROOT file")
        (self.version,) = struct.unpack_from(">i", d, 4)
        big = self.version >= 1000000
        (self.begin,) = struct.unpack_from(">i", d, 8)
        if big:
            self.end, self.seek_free = struct.unpack_from(">qq", d, 12)
            p = 28
        else:
            self.end, self.seek_free = struct.unpack_from(">ii", d, 12)
            p = 20
        self.nbytes_free, self.nfree, self.nbytes_name = struct.unpack_from(">iii", d, p)
        p += 12
        self.units = d[p]
        (self.compress,) = struct.unpack_from(">i", d, p + 1)
        if not 0 < self.begin < len(d):
            raise RootFormatError(f"{self.path}: header fBEGIN {self.begin} outside the file")
        # an unclosed file keeps the header written at creation: fEND is not
        # the file size and the top directory has no keys list
        self.closed = self.end == len(d)
        self.top = self._dir_record(self.begin + self.nbytes_name)

    # -- records -------------------------------------------------------------
    @_checked
    def read_key(self, pos: int) -> Key:
        d = self.data
        if pos < 0 or pos + 18 > len(d):
            raise RootFormatError(f"{self.path}: key at {pos} outside the file")
        nbytes, version, objlen, _datime, keylen, cycle = struct.unpack_from(">ihiIhh", d, pos)
        p = pos + 18
        if version > 1000:
            seek_key, seek_pdir = struct.unpack_from(">qq", d, p)
            p += 16
        else:
            seek_key, seek_pdir = struct.unpack_from(">ii", d, p)
            p += 8
        cls, p = _tstring(d, p)
        name, p = _tstring(d, p)
        title, p = _tstring(d, p)
        return Key(pos, nbytes, version, objlen, keylen, cycle, seek_key, seek_pdir, cls, name, title, p)

    def _dir_record(self, pos: int) -> dict:
        d = self.data
        if not 0 <= pos <= len(d) - 18:
            raise RootFormatError(f"{self.path}: directory record at {pos} outside the file")
        version, _c, _m, nbytes_keys, nbytes_name = struct.unpack_from(">hIIii", d, pos)
        p = pos + 18
        if version > 1000:
            seek_dir, seek_parent, seek_keys = struct.unpack_from(">qqq", d, p)
        else:
            seek_dir, seek_parent, seek_keys = struct.unpack_from(">iii", d, p)
        return {"seek_dir": seek_dir, "seek_parent": seek_parent, "seek_keys": seek_keys,
                "nbytes_keys": nbytes_keys}

    def _keys_list(self, rec: dict) -> list[Key]:
        if rec["seek_keys"] <= 0:
            raise RootFormatError(
                f"{self.path}: directory without a keys list (file not closed: header fEND "
                f"{self.end}, file size {len(self.data)})")
        head = self.read_key(rec["seek_keys"])
        p = rec["seek_keys"] + head.keylen
        (n,) = struct.unpack_from(">i", self.data, p)
        p += 4
        keys = []
        for _ in range(n):
            k = self.read_key(p)
            keys.append(k)
            p = k.header_end
        return keys

    @_checked
    def keys(self, directory: str = "") -> list[Key]:
        """Keys of a directory ("" = top, "A/B" = nested)."""
        rec = self.top
        for part in [s for s in directory.split("/") if s]:
            k = self._find(self._keys_list(rec), part)
            if not k.class_name.startswith("TDirectory"):
                raise RootFormatError(f"{self.path}: {part} is a {k.class_name}, not a directory")
            rec = self._dir_record(k.seek_key + k.keylen)
        return self._keys_list(rec)

    def _find(self, keys: list[Key], name: str) -> Key:
        hits = [k for k in keys if k.name == name]
        if not hits:
            raise KeyError(f"{self.path}: no object named {name!r}")
        return max(hits, key=lambda k: k.cycle)

    @_checked
    def get_key(self, path: str) -> Key:
        """Key of the highest cycle of ``dir/.../name``."""
        parts = [s for s in path.split("/") if s]
        return self._find(self.keys("/".join(parts[:-1])), parts[-1])

    @_checked
    def payload(self, key: Key) -> bytes:
        """The record's object bytes, decompressed (ObjLen bytes)."""
        start = key.seek_key + key.keylen
        if key.seek_key < 0 or key.keylen < 0 or key.nbytes < key.keylen or key.seek_key + key.nbytes > len(self.data):
            raise RootFormatError(f"{self.path}: record {key.name} lies outside the file")
        raw = self.data[start:key.seek_key + key.nbytes]
        if not key.compressed:
            return raw
        out = []
        got = 0
        p = 0
        while got < key.objlen:
            if p + 9 > len(raw):
                raise RootFormatError(f"{self.path}: {key.name}: truncated compressed block")
            alg = raw[p:p + 2]
            csize = raw[p + 3] | raw[p + 4] << 8 | raw[p + 5] << 16
            usize = raw[p + 6] | raw[p + 7] << 8 | raw[p + 8] << 16
            block = raw[p + 9:p + 9 + csize]
            if alg == b"ZL":
                part = zlib.decompress(block)
            elif alg == b"XZ":
                part = lzma.decompress(block)
            else:
                raise RootFormatError(
                    f"{self.path}: {key.name}: compression {alg!r} is not supported (zlib and LZMA are)")
            if len(part) != usize:
                raise RootFormatError(f"{self.path}: {key.name}: block inflated to {len(part)}, not {usize}")
            out.append(part)
            got += usize
            p += 9 + csize
        res = b"".join(out)
        if len(res) != key.objlen:
            raise RootFormatError(f"{self.path}: {key.name}: {len(res)} bytes inflated, ObjLen {key.objlen}")
        return res

    def walk(self):
        """Every key from fBEGIN to the end of the data, in file order (free
        gaps, which carry a negative length, are stepped over)."""
        pos = self.begin
        stop = len(self.data)
        while pos + 4 <= stop:
            (n,) = struct.unpack_from(">i", self.data, pos)  # in range: pos + 4 <= stop
            if n < 0:
                pos -= n
                continue
            if n == 0:
                break
            k = self.read_key(pos)
            yield k
            pos += n

    # -- objects -------------------------------------------------------------
    @_checked
    def tree(self, path: str) -> "Tree":
        key = self.get_key(path)
        if key.class_name != "TTree":
            raise RootFormatError(f"{self.path}: {path} is a {key.class_name}, not a TTree")
        return Tree(self, key)

    @_checked
    def graph(self, path: str):
        """(fX, fY, fBits) of a TGraph."""
        key = self.get_key(path)
        if key.class_name != "TGraph":
            raise RootFormatError(f"{self.path}: {path} is a {key.class_name}, not a TGraph")
        buf = self.payload(key)
        p, bits = _skip_named_and_attributes(buf, path)
        (n,) = struct.unpack_from(">i", buf, p)
        p += 4
        arrays = []
        for name in ("fX", "fY"):
            present = buf[p]
            p += 1
            if not present:
                arrays.append(np.zeros(0))
                continue
            if p + 8 * n > len(buf):
                raise RootFormatError(f"{self.path}: {path} {name} runs past the record")
            arrays.append(np.frombuffer(buf, dtype=">f8", count=n, offset=p).astype(np.float64))
            p += 8 * n
        return arrays[0], arrays[1], bits


    @_checked
    def th1_stats(self, path: str) -> dict:
        """Fill statistics of a 1-D histogram (TH1D/TH1F/TH1I): after the
        class header, TH1's header, TNamed and the three attribute bases come
        fNcells, the three axes (skipped by their byte counts), fBarOffset,
        fBarWidth, then fEntries, fTsumw, fTsumw2, fTsumwx, fTsumwx2.
        Returns those with mean = sumwx / sumw and rms = sqrt(|sumwx2 / sumw -
        mean^2|), as TH1::GetMean / GetRMS report them."""
        key = self.get_key(path)
        if not key.class_name.startswith("TH1"):
            raise RootFormatError(f"{self.path}: {path} is a {key.class_name}, not a 1-D histogram")
        buf = self.payload(key)
        p = 12  # the class's and TH1's byte counts and versions
        for base in ("TNamed", "TAttLine", "TAttFill", "TAttMarker"):
            p = _skip_streamed(buf, p, f"{path} {base}")
        (ncells,) = struct.unpack_from(">i", buf, p)
        p += 4
        for axis in ("fXaxis", "fYaxis", "fZaxis"):
            p = _skip_streamed(buf, p, f"{path} {axis}")
        p += 4  # fBarOffset, fBarWidth
        entries, sumw, sumw2, sumwx, sumwx2 = struct.unpack_from(">5d", buf, p)
        mean = sumwx / sumw if sumw else 0.0
        rms = float(np.sqrt(abs(sumwx2 / sumw - mean * mean))) if sumw else 0.0
        return {"ncells": ncells, "entries": entries, "sumw": sumw, "sumw2": sumw2, "sumwx": sumwx,
                "sumwx2": sumwx2, "mean": mean, "rms": rms}


class Tree:
    """Branch columns of one TTree, gathered from its basket keys."""

    @_checked
    def __init__(self, f: RootFile, key: Key):
        self.file = f
        self.key = key
        self.name = key.name
        buf = f.payload(key)
        p, _bits = _skip_named_and_attributes(buf, f"TTree {key.name}")
        (self.entries,) = struct.unpack_from(">q", buf, p)
        self._baskets: dict[str, list[Basket]] = {}
        for k in f.walk():
            if k.class_name == "TBasket" and k.title == self.name:
                _v, _bs, nbs, nev, last, _flag = struct.unpack_from(">hiiiib", f.data, k.header_end)
                self._baskets.setdefault(k.name, []).append(Basket(k, nev, nbs, last))

    def branch_names(self) -> list[str]:
        return sorted(self._baskets)

    def _branch(self, name: str) -> list[Basket]:
        if name not in self._baskets:
            raise KeyError(f"{self.file.path}: tree {self.name} has no baskets of branch {name!r}")
        bs = self._baskets[name]
        total = sum(b.nev_buf for b in bs)
        if total != self.entries:
            raise RootFormatError(
                f"{self.file.path}: branch {name} holds {total} entries in its basket keys, tree {self.name} "
                f"has {self.entries} (baskets kept inside the tree record, or two trees named {self.name})")
        return bs

    def _entry_spans(self, b: Basket, buf: bytes):
        """(start, end) of every entry of a basket in its payload."""
        kl = b.key.keylen
        data_len = b.last - kl
        if data_len < 0 or data_len > len(buf):
            raise RootFormatError(f"{self.file.path}: basket of {b.key.name}: Last {b.last} outside the buffer")
        if data_len == len(buf):
            return None  # fixed-size entries: no offsets array
        (cnt,) = struct.unpack_from(">i", buf, data_len)
        if cnt < b.nev_buf:
            raise RootFormatError(f"{self.file.path}: basket of {b.key.name}: {cnt} offsets for {b.nev_buf} entries")
        offs = np.frombuffer(buf, dtype=">i4", count=b.nev_buf, offset=data_len + 4).astype(np.int64) - kl
        ends = np.append(offs[1:], data_len)
        if b.nev_buf and (offs[0] < 0 or (ends < offs).any() or ends[-1] > data_len):
            raise RootFormatError(f"{self.file.path}: basket of {b.key.name}: entry offsets out of order or range")
        return list(zip(offs.tolist(), ends.tolist()))

    @_checked
    def array(self, name: str, dtype) -> np.ndarray:
        """A branch of one fixed-size value per entry (a leaf such as
        ``x/D``, ``x/F``, ``x/I``); ``dtype`` is the value's numpy type,
        as SetBranchAddress takes the caller's C type."""
        dt = np.dtype(dtype).newbyteorder(">")
        parts = []
        for b in self._branch(name):
            buf = self.file.payload(b.key)
            if self._entry_spans(b, buf) is not None:
                raise RootFormatError(f"{self.file.path}: branch {name} has entries of varying size")
            if b.last - b.key.keylen != b.nev_buf * dt.itemsize:
                raise RootFormatError(
                    f"{self.file.path}: branch {name}: {b.last - b.key.keylen} bytes for {b.nev_buf} "
                    f"entries of {dt.itemsize} bytes")
            parts.append(np.frombuffer(buf, dtype=dt, count=b.nev_buf))
        return np.concatenate(parts).astype(dt.newbyteorder("="))

    @_checked
    def vectors(self, name: str, dtype=np.float64) -> list[np.ndarray]:
        """A ``std::vector<T>`` branch (entries of varying length): one
        numpy array per entry."""
        dt = np.dtype(dtype).newbyteorder(">")
        out = []
        for b in self._branch(name):
            buf = self.file.payload(b.key)
            spans = self._entry_spans(b, buf)
            if spans is None:
                raise RootFormatError(f"{self.file.path}: branch {name} has no entry offsets")
            for s, e in spans:
                (bc,) = struct.unpack_from(">I", buf, s)
                if not bc & BYTECOUNT_FLAG or s + 4 + (bc & ~BYTECOUNT_FLAG) != e:
                    raise RootFormatError(f"{self.file.path}: branch {name}: entry at {s} has a bad byte count")
                (n,) = struct.unpack_from(">i", buf, s + 6)
                if s + 10 + n * dt.itemsize != e:
                    raise RootFormatError(f"{self.file.path}: branch {name}: entry at {s} of {n} values "
                                          f"does not fill its {e - s} bytes")
                out.append(np.frombuffer(buf, dtype=dt, count=n, offset=s + 10).astype(dt.newbyteorder("=")))
        return out
