"""TMI container I/O: the reference's multimodal file format
(tfce_mediation/tm_io.py:72-450, ``write_tm_filetype`` / ``read_tm_filetype``),
which feeds the multisurface (mmr) path: subject data, masks, affines,
surfaces and adjacency sets in one file.

Layout: a text header (``tmi``; ``format binary_<byteorder>_endian 0.1`` or
``format ascii 0.1``; one block of lines per element: ``element <kind>``,
``dtype``, ``nbytes`` and kind-specific shape lines; ``history ...`` lines;
``end_header``) followed, in binary files, by the payloads.  The payloads
follow the header's element order except that the column ids precede the
adjacency objects (the reference writes them in that order while its header
lists them the other way round; its reader, which follows the header order,
misreads files holding both -- this reader follows the written order).
Arrays are stored transposed (Fortran order of the logical array), as the
reference writes them; adjacency sets are pickled Python objects.  A reader
finds the payloads at (file size - sum of nbytes), as the reference does.

Deviations from the reference, on purpose: a call's history list starts
from the ``tmi_history`` argument only (the reference's default list is
shared between calls of one process and grows), and errors raise instead of
calling ``exit()``.  Loading the pickled adjacency objects executes pickle:
read only files you trust (the reference has the same property).
"""
from __future__ import annotations

import os
import pickle
import sys
from time import gmtime, strftime

import numpy as np

VERSION = "0.1"


def tm_filetype_version():
    """tm_io.py:34-37."""
    return VERSION


def check_outname(outname):
    """pyfunc.py:315-326: an existing file name gets a ``new_`` prefix (and
    an existing ``new_`` file is replaced)."""
    if os.path.exists(outname):
        path, name = os.path.split(outname)
        outname = "new_%s" % name if not path else "%s/new_%s" % (path, name)
        print("Output file aleady exists. Renaming output file to %s" % outname)
        if os.path.exists(outname):
            print("%s also exists. Overwriting the file." % outname)
            os.remove(outname)
    return outname


def _count(arr, one_ndim, many_ndim):
    """Number of objects in an element argument: a single array of
    `one_ndim` dimensions, or a stack / object array of them."""
    if isinstance(arr, (list, tuple)) and arr and all(isinstance(x, np.ndarray) for x in arr):
        return len(arr)  # a list of arrays (their shapes may differ)
    a = np.asarray(arr) if not isinstance(arr, np.ndarray) else arr
    if a.dtype.kind == "O" or a.ndim == many_ndim:
        return int(a.shape[0])
    if a.ndim == one_ndim:
        return 1
    raise ValueError("element dimensions are not understood")


def _items(arr, n, one_ndim):
    if isinstance(arr, (list, tuple)) and arr and all(isinstance(x, np.ndarray) for x in arr):
        return list(arr)
    a = np.asarray(arr) if not isinstance(arr, np.ndarray) else arr
    if n == 1 and a.dtype.kind != "O" and a.ndim == one_ndim:
        return [a]
    return [a[i] for i in range(n)]


def _empty(x):
    return x is None or (isinstance(x, list) and len(x) == 0)


def write_tm_filetype(outname, columnids=[], imgtype=[], checkname=True, output_binary=True, image_array=[],
                      masking_array=[], maskname=[], affine_array=[], vertex_array=[], face_array=[], surfname=[],
                      adjacency_array=[], tmi_history=None, append_history=True):
    """Write a TMI file (tm_io.py:72-281): image_array (V, n) float32 data,
    masking_array 3-D boolean mask(s), affine_array 4x4 matrices,
    vertex_array / face_array surfaces (with surfname), adjacency_array
    adjacency sets, columnids, and the history lines (tmi_history plus, with
    append_history, a ``history mode_add`` line for what this call adds).
    Returns the file name written."""
    history = list(tmi_history or [])
    counted = [0, 0, 0, 0]  # masks, affines, objects, adjacency sets already recorded in the history
    for line in history:
        f = line.split(" ")
        sign = {"mode_add": 1, "mode_sub": -1}.get(f[1], 0)
        if f[1] not in ("mode_add", "mode_sub", "mode_replace", "mode_reorder"):
            print("Error reading history. Mode %s is not understood. Count is reflect number of element in "
                  "current file" % f[1])
        for j in range(4):
            counted[j] += sign * int(f[4 + j]) if sign else 0

    masks = [] if _empty(masking_array) else _items(masking_array, _count(masking_array, 3, 4), 3)
    affines = [] if _empty(affine_array) else _items(affine_array, _count(affine_array, 2, 3), 2)
    verts = [] if _empty(vertex_array) else _items(vertex_array, _count(vertex_array, 2, 3), 2)
    faces = [] if _empty(face_array) else _items(face_array, len(verts), 2)
    if _empty(adjacency_array):
        adjs = []
    else:
        adj = np.asarray(adjacency_array, dtype=object) if not isinstance(adjacency_array, np.ndarray) \
            else adjacency_array
        adjs = [adj] if (adj.dtype.kind != "O" and adj.ndim == 1) else [adj[i] for i in range(adj.shape[0])]
    data = None if _empty(image_array) else np.asarray(image_array)
    cols = None if (isinstance(columnids, list) and len(columnids) == 0) else np.asarray(columnids)

    if not outname.endswith("tmi"):
        outname += ".tmi" if output_binary else ".ascii.tmi"
    if checkname:
        outname = check_outname(outname)

    head = ["tmi"]
    head.append("format binary_%s_endian %s" % (sys.byteorder, VERSION) if output_binary
                else "format ascii %s" % VERSION)
    head.append("comment made with TFCE_mediation")
    if data is not None:
        nvert, nsub = (len(data), 1) if data.ndim == 1 else data.shape[:2]
        head += ["element data_array", "dtype float32", "nbytes %d" % data.astype(np.float32).nbytes,
                 "datashape %d %d" % (nvert, nsub)]
    for i, m in enumerate(masks):
        m = np.asarray(m)
        head += ["element masking_array", "dtype uint8", "nbytes %d" % m.nbytes,
                 "nmasked %d" % int(np.count_nonzero(m)), "maskshape %d %d %d" % m.shape[:3],
                 "maskname %s" % (maskname[i] if i < len(maskname) else "unknown")]
    for a in affines:
        a = np.asarray(a)
        head += ["element affine", "dtype float32", "nbytes %d" % a.astype(np.float32).nbytes,
                 "affineshape %d %d" % a.shape[:2]]
    for i, (v, f) in enumerate(zip(verts, faces)):
        v, f = np.asarray(v), np.asarray(f)
        head += ["surfname %s" % (surfname[i] if i < len(surfname) else "unknown"),
                 "element vertex", "dtype float32", "nbytes %d" % v.astype(np.float32).nbytes,
                 "vertexshape %d %d" % v.shape[:2],
                 "element face", "dtype uint32", "nbytes %d" % f.astype(np.uint32).nbytes,
                 "faceshape %d %d" % f.shape[:2]]
    for a in adjs:
        head += ["element adjacency_object", "dtype python_object",
                 "nbytes %d" % len(pickle.dumps(a, -1)), "adjlength %d" % len(a)]
    if cols is not None:
        head += ["element column_id", "dtype %s" % cols.dtype, "nbytes %d" % cols.nbytes,
                 "listlength %d" % len(cols)]
    if append_history:
        now = int(strftime("%Y%m%d%H%M%S", gmtime()))
        history.append("history mode_add %d %d %d %d %d %d" % (
            now, 0 if data is None else 1, len(masks) - counted[0], len(affines) - counted[1],
            len(verts) - counted[2], len(adjs) - counted[3]))
    head += history
    head.append("end_header")
    with open(outname, "w") as o:
        o.write("\n".join(head) + "\n")

    if output_binary:
        with open(outname, "ab") as o:
            if data is not None:
                np.asarray(data.T, dtype=np.float32).tofile(o)
            for m in masks:
                np.asarray((np.asarray(m) * 1).T, dtype=np.uint8).tofile(o)
            for a in affines:
                np.asarray(np.asarray(a).T, dtype=np.float32).tofile(o)
            for v, f in zip(verts, faces):
                np.asarray(np.asarray(v).T, dtype=np.float32).tofile(o)
                np.asarray(np.asarray(f).T, dtype=np.uint32).tofile(o)
            if cols is not None:
                cols.tofile(o)
            for a in adjs:
                pickle.dump(a, o, protocol=pickle.HIGHEST_PROTOCOL)
    else:
        with open(outname, "a") as o:
            if data is not None:
                np.savetxt(o, data.astype(np.float32))
            for m in masks:
                x, y, z = np.nonzero(np.asarray(m))
                for i in range(len(x)):
                    o.write("%d %d %d\n" % (int(x[i]), int(y[i]), int(z[i])))
            for a in affines:
                np.savetxt(o, np.asarray(a).astype(np.float32))
            if cols is not None:
                cols.tofile(o, sep="\n", format="%s")
            for v, f in zip(verts, faces):
                for row in np.asarray(v):
                    o.write("%1.6f %1.6f %1.6f\n" % (row[0], row[1], row[2]))
                for row in np.asarray(f):
                    o.write("%d %d %d\n" % (int(row[0]), int(row[1]), int(row[2])))
    return outname


def read_tm_filetype(tm_file, verbose=True):
    """Read a TMI file (tm_io.py:284-448).  Returns the reference's tuple:
    (element, image_array, masking_array, maskname, affine_array,
    vertex_array, face_array, surfname, adjacency_array, tmi_history,
    columnids) -- lists of arrays, element the element kinds in file order."""
    filesize = os.stat(tm_file).st_size
    elems = []  # dicts: kind, dtype, nbytes (+ shape fields)
    shapes = {"datashape": [], "maskshape": [], "affineshape": [], "vertexshape": [], "faceshape": []}
    nmasked, maskname, surfname, adjlength, history = [], [], [], [], []
    listlength = 0
    with open(tm_file, "rb") as obj:
        first = obj.readline().decode("UTF-8").split()
        if not first or first[0] != "tmi":
            raise ValueError("not a TFCE_mediation image: %s" % tm_file)
        fmt = obj.readline().decode("UTF-8").split()
        if not fmt or fmt[0] != "format":
            raise ValueError("unknown reading file format")
        filetype = fmt[1]
        while True:
            words = obj.readline().decode("UTF-8").split()
            if not words:
                continue
            key = words[0]
            if key == "end_header":
                break
            if key == "element":
                elems.append({"kind": words[1]})
            elif key == "dtype":
                elems[-1]["dtype"] = words[1]
            elif key == "nbytes":
                elems[-1]["nbytes"] = int(words[1])
            elif key in shapes:
                shapes[key].append([int(w) for w in words[1:]])
            elif key == "nmasked":
                nmasked.append(int(words[1]))
            elif key == "maskname":
                maskname.append(words[1])
            elif key == "surfname":
                surfname.append(words[1])
            elif key == "adjlength":
                adjlength.append(int(words[1]))
            elif key == "history":
                history.append(" ".join(words))
            elif key == "listlength":
                listlength = int(words[1])
        out = {k: [] for k in ("data", "mask", "affine", "vertex", "face", "adj", "cols")}
        cnt = {k: 0 for k in ("mask", "affine", "vertex", "face", "adj")}

        def fortran(arr, shape):
            n = int(np.prod(shape))
            return np.asarray(arr[:n]).reshape(tuple(reversed(shape))).T

        if filetype.startswith("binary"):
            pos = filesize - sum(e["nbytes"] for e in elems)
            # written order: column ids before the adjacency objects
            order = [e for e in elems if e["kind"] != "adjacency_object"] + \
                [e for e in elems if e["kind"] == "adjacency_object"]
            for e in order:
                obj.seek(pos)
                if verbose:
                    print(pos)
                    print("reading %s" % e["kind"])
                kind = e["kind"]
                if kind == "adjacency_object":
                    obj_read = pickle.load(obj)
                    out["adj"].append(np.array(obj_read[:adjlength[cnt["adj"]]], dtype=object)
                                      if isinstance(obj_read, (list, np.ndarray)) else obj_read)
                    cnt["adj"] += 1
                else:
                    arr = np.fromfile(obj, dtype=e["dtype"], count=e["nbytes"] // np.dtype(e["dtype"]).itemsize)
                    if kind == "data_array":
                        out["data"].append(fortran(arr, shapes["datashape"][0]))
                    elif kind == "masking_array":
                        out["mask"].append(fortran(arr, shapes["maskshape"][cnt["mask"]]).astype(bool))
                        cnt["mask"] += 1
                    elif kind == "affine":
                        out["affine"].append(fortran(arr, shapes["affineshape"][cnt["affine"]]))
                        cnt["affine"] += 1
                    elif kind == "vertex":
                        out["vertex"].append(fortran(arr, shapes["vertexshape"][cnt["vertex"]]))
                        cnt["vertex"] += 1
                    elif kind == "face":
                        out["face"].append(fortran(arr, shapes["faceshape"][cnt["face"]]))
                        cnt["face"] += 1
                    elif kind == "column_id":
                        out["cols"].append(np.asarray(arr[:listlength]))
                pos += e["nbytes"]
        elif filetype == "ascii":
            for e in elems:
                kind = e["kind"]
                if kind == "data_array":
                    nv, ns = shapes["datashape"][0]
                    rows = [np.array(obj.readline().split(), dtype=np.float32) for _ in range(nv)]
                    out["data"].append(np.asarray(rows, dtype=np.float32).reshape(nv, ns))
                elif kind == "masking_array":
                    idx = np.array([obj.readline().split() for _ in range(nmasked[cnt["mask"]])], dtype=np.int64)
                    m = np.zeros(shapes["maskshape"][cnt["mask"]], bool)
                    if idx.size:
                        m[idx[:, 0], idx[:, 1], idx[:, 2]] = True
                    out["mask"].append(m)
                    cnt["mask"] += 1
                elif kind in ("affine", "vertex", "face"):
                    sh = shapes[kind + "shape"][cnt[kind]]
                    dt = np.int32 if kind == "face" else np.float32
                    out[kind].append(np.array([obj.readline().split() for _ in range(sh[0])], dtype=dt))
                    cnt[kind] += 1
                elif kind == "column_id":
                    out["cols"].append(np.array([obj.readline().strip().decode("UTF-8")
                                                 for _ in range(listlength)], dtype=e["dtype"]))
        else:
            raise ValueError("unknown filetype: %s" % filetype)
    return ([e["kind"] for e in elems], out["data"], out["mask"], maskname, out["affine"], out["vertex"],
            out["face"], surfname, out["adj"], history, out["cols"])
