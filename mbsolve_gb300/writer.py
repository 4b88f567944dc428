"""Result writers with the reference's writer interface
(mbsolve-lib/include/mbsolve/lib/writer.hpp:42-115, writer.cpp:26-60).

`writer.create_instance(name).write(file, results, dev, scen)` stores the
results of one simulation. The reference's only writer is HDF5
(writer-hdf5/src/writer_hdf5.cpp:31-110): global attributes timestep_size,
gridpoint_size, sim_endtime and dev_length, then one group per result with
a boolean attribute is_complex and datasets real (and imag when complex),
each rows x cols (FP64). The "npz" writer here keeps exactly that layout
in a numpy archive (keys "timestep_size", ..., "<result>/real",
"<result>/imag", "<result>/is_complex"), since no HDF5 library is
available to this package; the "hdf5" writer registers itself only when
h5py can be imported and then writes the reference's file layout.
"""
import numpy as np

_bootstraps = {}


class writer:
    """Base class and factory (writer.hpp:42-115)."""

    def __init__(self, name, extension):
        self._name = name
        self._ext = extension

    @staticmethod
    def get_avail_writers():
        return sorted(_bootstraps)

    @staticmethod
    def register_bootstrap(name, bootstrap):
        if name in _bootstraps:
            raise ValueError("Writer already registered.")
        _bootstraps[name] = bootstrap

    @staticmethod
    def register_writer(name, cls):
        writer.register_bootstrap(name, cls)

    @staticmethod
    def create_instance(name):
        if name not in _bootstraps:
            raise ValueError("Unknown writer " + name)
        return _bootstraps[name]()

    def get_name(self):
        return self._name

    def get_extension(self):
        return self._ext

    def write(self, file, results, dev, scen):
        raise NotImplementedError


def _global_attrs(dev, scen):
    return {"timestep_size": scen.get_timestep_size(),
            "gridpoint_size": scen.get_gridpoint_size(),
            "sim_endtime": scen.get_endtime(),
            "dev_length": dev.get_length()}


class writer_npz(writer):
    """The HDF5 writer's layout in a numpy .npz archive."""

    def __init__(self):
        super().__init__("npz", "npz")

    def write(self, file, results, dev, scen):
        out = {k: np.float64(v) for k, v in _global_attrs(dev, scen).items()}
        for r in results:
            name = r.get_name()
            shape = (r.get_rows(), r.get_cols())
            out[name + "/is_complex"] = np.bool_(r.is_complex())
            out[name + "/real"] = np.asarray(r.get_data_real(),
                                             dtype=np.float64).reshape(shape)
            if r.is_complex():
                out[name + "/imag"] = np.asarray(r.get_data_imag(),
                                                 dtype=np.float64).reshape(shape)
        with open(file, "wb") as f:
            np.savez(f, **out)


def read_npz(file):
    """{attr: float, result name: {"is_complex", "real", ["imag"]}}."""
    z = np.load(file)
    out = {}
    for k in z.files:
        if "/" in k:
            name, field = k.rsplit("/", 1)
            out.setdefault(name, {})[field] = z[k] if field != "is_complex" else bool(z[k])
        else:
            out[k] = float(z[k])
    return out


writer.register_writer("npz", writer_npz)

try:  # the reference's own format, where h5py exists
    import h5py as _h5py

    class writer_hdf5(writer):
        """writer_hdf5.cpp:31-110 through h5py."""

        def __init__(self):
            super().__init__("hdf5", "hdf")

        def write(self, file, results, dev, scen):
            with _h5py.File(file, "w") as f:
                for k, v in _global_attrs(dev, scen).items():
                    f.attrs[k] = np.float64(v)
                for r in results:
                    g = f.create_group(r.get_name())
                    g.attrs["is_complex"] = bool(r.is_complex())
                    shape = (r.get_rows(), r.get_cols())
                    g.create_dataset("real", data=np.asarray(
                        r.get_data_real(), dtype=np.float64).reshape(shape))
                    if r.is_complex():
                        g.create_dataset("imag", data=np.asarray(
                            r.get_data_imag(), dtype=np.float64).reshape(shape))

    writer.register_writer("hdf5", writer_hdf5)
except ImportError:
    pass
