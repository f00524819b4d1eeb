"""Saving and loading clustering estimators.

The reference stores estimators with ``obj.save(file_name, model_name)`` and
restores them with ``pyemma.load(file_name, model_name)``
(pyemma/_base/serialization/serialization.py:212-290): the parameters and the
fields each class lists (``initial_centers_`` and ``_converged`` for k-means,
kmeans.py:49-50; ``_dtrajs``, ``_previous_stride``, ``_index_states``,
``_overwrite_dtrajs``, interface.py:71) go into an HDF5 file that can hold
several models.  h5py is not part of this package's environment, so the
container here is a NumPy ``.npz`` archive with the same role: several named
models per file, parameters as JSON, arrays as arrays, nothing pickled (the
file is read with ``allow_pickle=False``).  The data source is not saved
(the reference's ``save_streaming_chain=False``); a loaded estimator keeps
its centers, its model fields and the dtrajs it had computed.
"""
import json
import os

import numpy as np

__all__ = ["save", "load", "list_models"]

# model fields saved beside the parameters, when the object has them
_FIELDS = ("initial_centers_", "_converged", "_dtrajs", "_previous_stride", "_index_states", "_overwrite_dtrajs",
           "inertias", "n_iter", "_estimated")
_LIST_FIELDS = ("_dtrajs", "_index_states")


def _classes():
    from .coordinates import clustering as cl
    return {c.__name__: c for c in (cl.KmeansClustering, cl.MiniBatchKmeansClustering, cl.RegularSpaceClustering,
                                    cl.UniformTimeClustering, cl.AssignCenters)}


def _plain(value):
    if isinstance(value, (np.bool_, bool)):
        return bool(value)
    if isinstance(value, np.integer):
        return int(value)
    if isinstance(value, np.floating):
        return float(value)
    return value


def _read(file_name):
    if not os.path.exists(file_name):
        return {}
    with np.load(file_name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def list_models(file_name):
    """Names of the models stored in file_name."""
    return sorted({k.split("/", 1)[0] for k in _read(file_name) if k.endswith("/__class__")})


def save(obj, file_name, model_name="default", overwrite=False, save_streaming_chain=False):
    """Stores obj's parameters and model fields in file_name under model_name.

    Other models in the file are kept.  An existing model of that name is
    replaced only with overwrite=True, else RuntimeError.
    save_streaming_chain is accepted for the reference's signature; the data
    source is never stored."""
    if "/" in model_name or not model_name:
        raise ValueError("model_name must be a non-empty name without '/', got %r" % (model_name,))
    if type(obj).__name__ not in _classes():
        raise TypeError("cannot save objects of type %s" % type(obj).__name__)
    entries = _read(file_name)
    prefix = model_name + "/"
    if any(k.startswith(prefix) for k in entries):
        if not overwrite:
            raise RuntimeError('model "%s" is already stored in %s; pass overwrite=True or use another name'
                               % (model_name, file_name))
        entries = {k: v for k, v in entries.items() if not k.startswith(prefix)}
    params, fields = {}, {}
    for name, value in obj.get_params().items():
        if isinstance(value, np.ndarray):
            entries[prefix + "param/" + name] = value
        else:
            params[name] = _plain(value)
    for name in _FIELDS:
        if not hasattr(obj, name):
            continue
        value = getattr(obj, name)
        if name in _LIST_FIELDS:
            value = list(value)
            fields[name] = {"list": len(value)}
            for i, a in enumerate(value):
                entries["%sfield/%s/%d" % (prefix, name, i)] = np.asarray(a)
        elif isinstance(value, np.ndarray):
            entries[prefix + "field/" + name] = value
        else:
            fields[name] = {"value": _plain(value)}
    entries[prefix + "__class__"] = np.array(type(obj).__name__)
    entries[prefix + "__params__"] = np.array(json.dumps(params))
    entries[prefix + "__fields__"] = np.array(json.dumps(fields))
    tmp = file_name + ".tmp"
    with open(tmp, "wb") as f:
        np.savez(f, **entries)
    os.replace(tmp, file_name)


def load(file_name, model_name="default"):
    """The estimator stored in file_name under model_name."""
    import inspect
    entries = _read(file_name)
    prefix = model_name + "/"
    if prefix + "__class__" not in entries:
        raise KeyError('no model "%s" in %s (models: %s)' % (model_name, file_name, list_models(file_name)))
    cls = _classes()[str(entries[prefix + "__class__"])]
    params = json.loads(str(entries[prefix + "__params__"]))
    for key, value in entries.items():
        if key.startswith(prefix + "param/"):
            params[key[len(prefix + "param/"):]] = value
    accepted = set(inspect.signature(cls.__init__).parameters) - {"self"}
    obj = cls(**{k: v for k, v in params.items() if k in accepted})
    # every parameter once more: some constructors fix one (mini-batch k-means
    # draws its own seed), and the saved value is the one to restore
    obj.set_params(**params)
    fields = json.loads(str(entries[prefix + "__fields__"]))
    for name, spec in fields.items():
        if "list" in spec:
            setattr(obj, name, [entries["%sfield/%s/%d" % (prefix, name, i)] for i in range(spec["list"])])
        else:
            setattr(obj, name, spec["value"])
    for key, value in entries.items():
        if key.startswith(prefix + "field/") and key.count("/") == 2:
            setattr(obj, key[len(prefix + "field/"):], value)
    return obj
