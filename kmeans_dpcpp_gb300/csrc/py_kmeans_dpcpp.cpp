// pybind11 module `_kmeans_dpcpp`: the Python surface of kmeans_dpcpp
// (python_api/_kmeans_lloyd.cpp:1277-1449) on top of the GB300 C ABI
// (include/kmeans_gb300.h).
//
// Mirrors, function by function, the reference wrappers: the same names,
// argument names and order, the same shape / dtype / contiguity checks in the
// same order and with the same ValueError messages, and the same return
// values.  What changes is the array and queue model:
//   * arrays are any objects exposing __cuda_array_interface__ (torch CUDA
//     tensors, CuPy arrays, ...) instead of dpctl usm_ndarray;
//   * `sycl_queue` is a CUDA stream: None (legacy default stream), an int
//     handle, or an object with a `cuda_stream` attribute (torch.cuda.Stream);
//   * the returned (host_task_event, compute_event) pair are Event objects
//     with .wait(); the first keeps the argument arrays alive until waited on,
//     like dpctl::utils::keep_args_alive;
//   * `depends` is a list of such Event objects.
// No CUDA headers are needed here: every device operation goes through the
// C ABI.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "kmeans_gb300.h"

namespace py = pybind11;

namespace {

enum class DT { F32, F64, I32, I64, OTHER };

struct Arr {
    void *ptr = nullptr;
    std::vector<int64_t> shape;
    DT dt = DT::OTHER;
    bool c_contig = true;
    py::object owner;

    int ndim() const { return (int)shape.size(); }
    int64_t size() const {
        int64_t s = 1;
        for (auto v : shape) s *= v;
        return s;
    }
    int64_t get_shape(int i) const { return shape.at(i); }
    template <typename T>
    T *data() const { return static_cast<T *>(ptr); }
};

DT dt_of(const std::string &ts) {
    if (ts.size() < 3) return DT::OTHER;
    std::string body = ts.substr(1);
    if (ts[0] == '>') return DT::OTHER;
    if (body == "f4") return DT::F32;
    if (body == "f8") return DT::F64;
    if (body == "i4") return DT::I32;
    if (body == "i8") return DT::I64;
    return DT::OTHER;
}

int64_t item_size(DT d) { return (d == DT::F32 || d == DT::I32) ? 4 : 8; }

Arr as_arr(const py::object &o) {
    if (!py::hasattr(o, "__cuda_array_interface__"))
        throw py::type_error("expected a CUDA array (an object exposing __cuda_array_interface__)");
    py::dict cai = o.attr("__cuda_array_interface__");
    Arr a;
    a.owner = o;
    for (auto v : cai["shape"].cast<py::tuple>()) a.shape.push_back(v.cast<int64_t>());
    a.dt = dt_of(cai["typestr"].cast<std::string>());
    py::tuple data = cai["data"].cast<py::tuple>();
    a.ptr = reinterpret_cast<void *>(data[0].cast<uintptr_t>());
    if (cai.contains("strides") && !cai["strides"].is_none()) {
        auto st = cai["strides"].cast<py::tuple>();
        int64_t expect = (a.dt == DT::OTHER) ? 0 : item_size(a.dt);
        if (a.dt == DT::OTHER) {
            std::string ts = cai["typestr"].cast<std::string>();
            expect = std::stoll(ts.substr(2));
        }
        for (int i = a.ndim() - 1; i >= 0; --i) {
            if (a.shape[i] != 1 && st[i].cast<int64_t>() != expect) a.c_contig = false;
            expect *= a.shape[i];
        }
    }
    return a;
}

template <std::size_t N>
bool all_c_contiguous(const Arr (&args)[N]) {
    for (auto &a : args)
        if (!a.c_contig) return false;
    return true;
}
template <std::size_t N>
bool same_typenum_as(DT t, const Arr (&args)[N]) {
    for (auto &a : args)
        if (a.dt != t) return false;
    return true;
}
bool is_1d(const Arr &a) { return a.ndim() == 1; }
bool is_2d(const Arr &a) { return a.ndim() == 2; }
bool is_3d(const Arr &a) { return a.ndim() == 3; }
bool is_0d(const Arr &a) { return a.size() == 1; }

// ---- the queue: a CUDA stream plus the device it runs on ----
struct Queue {
    kmc_stream_t stream = nullptr;
    int device = -1;
};

Queue as_queue(const py::object &q) {
    Queue r;
    if (q.is_none()) {
        r.stream = nullptr;
    } else if (py::isinstance<py::int_>(q)) {
        r.stream = reinterpret_cast<kmc_stream_t>(q.cast<uintptr_t>());
    } else if (py::hasattr(q, "cuda_stream")) {
        r.stream = reinterpret_cast<kmc_stream_t>(q.attr("cuda_stream").cast<uintptr_t>());
        if (py::hasattr(q, "device")) {
            py::object dev = q.attr("device");
            if (py::hasattr(dev, "index") && !dev.attr("index").is_none())
                r.device = dev.attr("index").cast<int>();
        }
    } else {
        throw py::type_error("sycl_queue must be None, an int stream handle or a CUDA stream object");
    }
    if (r.device < 0) {
        int d = 0;
        if (kmc_current_device(&d) != KMC_OK) throw std::runtime_error(kmc_last_error());
        r.device = d;
    }
    return r;
}

// Replaces queues_are_compatible (_kmeans_lloyd.cpp:46-56): every array must
// live on the stream's device.
template <std::size_t N>
bool queues_are_compatible(const Queue &q, const Arr (&arrs)[N]) {
    for (auto &a : arrs) {
        if (a.ptr == nullptr || a.size() == 0) continue;
        int dev = -1;
        if (kmc_pointer_device(a.ptr, &dev) != KMC_OK) return false;
        if (dev != q.device) return false;
    }
    return true;
}

// ---- events ----
struct EventHandle {
    kmc_event_t ev = nullptr;
    ~EventHandle() {
        if (ev) kmc_event_destroy(ev);
    }
};

struct Event {
    std::shared_ptr<EventHandle> h;
    py::list keep_alive;
    void wait() {
        if (h && h->ev) {
            int rc = kmc_event_synchronize(h->ev);
            if (rc != KMC_OK) throw std::runtime_error(kmc_last_error());
        }
        keep_alive = py::list();
    }
    bool is_complete() const {
        if (!h || !h->ev) return true;
        int done = 0;
        if (kmc_event_query(h->ev, &done) != KMC_OK) throw std::runtime_error(kmc_last_error());
        return done != 0;
    }
};

void check(int rc) {
    if (rc == KMC_OK) return;
    if (rc == KMC_ERR_INVALID_ARGUMENT) throw py::value_error(kmc_last_error());
    if (rc == KMC_ERR_OUT_OF_MEMORY) throw std::bad_alloc();
    throw std::runtime_error(kmc_last_error());
}

void wait_on(const Queue &q, const std::vector<Event> &depends) {
    for (auto &e : depends)
        if (e.h && e.h->ev) check(kmc_stream_wait_event(q.stream, e.h->ev));
}

template <std::size_t N>
std::pair<Event, Event> make_events(const Queue &q, const Arr (&keep)[N]) {
    auto h = std::make_shared<EventHandle>();
    check(kmc_event_create(&h->ev));
    check(kmc_event_record(h->ev, q.stream));
    Event ht, comp;
    ht.h = h;
    comp.h = h;
    for (auto &a : keep) ht.keep_alive.append(a.owner);
    return {ht, comp};
}

const char *kUnsupportedFloat =
    "Unsupported elemental data type. Expecting single or double precision floating point numbers";

// ---------------------------------------------------------------------------
// _kmeans_lloyd.cpp:60-105
std::pair<Event, Event> py_broadcast_divide(py::object Xo, py::object yo, size_t wgs,
                                            py::object qo, std::vector<Event> depends) {
    Arr X = as_arr(Xo), y = as_arr(yo);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_1d(y) || !all_c_contiguous({X, y}))
        throw py::value_error("Arguments must be a matrix and a vector with C-contiguous layout");
    if (y.get_shape(0) != X.get_shape(1))
        throw py::value_error(
            "Array dimensions of arguments are not consistent, X.shape[1] != y.shape[0]");
    if (!queues_are_compatible(q, {X, y}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    if (!same_typenum_as(y.dt, {X}))
        throw py::value_error("Arguments must have the same elemental data types.");
    wait_on(q, depends);
    if (y.dt == DT::F32)
        check(kmc_broadcast_divide_f32(X.data<float>(), y.data<float>(), X.get_shape(0),
                                       X.get_shape(1), (int64_t)wgs, q.stream));
    else if (y.dt == DT::F64)
        check(kmc_broadcast_divide_f64(X.data<double>(), y.data<double>(), X.get_shape(0),
                                       X.get_shape(1), (int64_t)wgs, q.stream));
    else
        throw py::value_error(kUnsupportedFloat);
    return make_events(q, {X, y});
}

// _kmeans_lloyd.cpp:108-152
std::pair<Event, Event> py_half_l2_norm_squared(py::object Xo, py::object yo, size_t wgs,
                                                py::object qo, std::vector<Event> depends) {
    Arr X = as_arr(Xo), y = as_arr(yo);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_1d(y) || !all_c_contiguous({X, y}))
        throw py::value_error("Arguments must be a matrix and a vector with C-contiguous layout");
    if (y.get_shape(0) != X.get_shape(1))
        throw py::value_error(
            "Array dimensions of arguments are not consistent, X.shape[1] != y.shape[0]");
    if (!queues_are_compatible(q, {X, y}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    if (!same_typenum_as(y.dt, {X}))
        throw py::value_error("Arguments must have the same elemental data types.");
    wait_on(q, depends);
    if (y.dt == DT::F32)
        check(kmc_half_l2_norm_squared_f32(X.data<float>(), y.data<float>(), X.get_shape(0),
                                           X.get_shape(1), (int64_t)wgs, q.stream));
    else if (y.dt == DT::F64)
        check(kmc_half_l2_norm_squared_f64(X.data<double>(), y.data<double>(), X.get_shape(0),
                                           X.get_shape(1), (int64_t)wgs, q.stream));
    else
        throw py::value_error(kUnsupportedFloat);
    return make_events(q, {X, y});
}

// _kmeans_lloyd.cpp:155-282
std::pair<Event, Event> py_reduce_centroids_data(py::object a0, py::object a1, py::object a2,
                                                 py::object a3, py::object a4, py::object a5,
                                                 size_t wgs, py::object qo,
                                                 std::vector<Event> depends) {
    Arr szc = as_arr(a0), cc = as_arr(a1), osz = as_arr(a2), oc = as_arr(a3), ol = as_arr(a4),
        one = as_arr(a5);
    Queue q = as_queue(qo);
    if (!is_2d(szc) || !is_3d(cc) || !is_1d(osz) || !is_2d(oc) || !is_1d(ol) || !is_1d(one))
        throw py::value_error("Array dimensions of inputs are not consistent");
    int64_t n_copies = szc.get_shape(0), n_clusters = szc.get_shape(1),
            n_features = cc.get_shape(1);
    if (n_copies != cc.get_shape(0) || n_clusters != cc.get_shape(2) ||
        n_clusters != osz.get_shape(0) || n_clusters != oc.get_shape(1) ||
        n_features != oc.get_shape(0) || n_clusters != ol.get_shape(0))
        throw py::value_error("Dimensions mismatch");
    DT dT = szc.dt, iT = one.dt;
    if (!same_typenum_as(dT, {cc, osz, oc}) || !same_typenum_as(iT, {ol}))
        throw py::value_error("Array element data types must be consisten");
    if (!all_c_contiguous({szc, cc, osz, oc, ol, one}))
        throw py::value_error("All array arguments must be C-contiguous");
    if (!queues_are_compatible(q, {szc, cc, osz, oc, ol, one}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    wait_on(q, depends);
#define RCD(SUF, T, I)                                                                        \
    check(kmc_reduce_centroids_data_##SUF(szc.data<T>(), cc.data<T>(), osz.data<T>(),        \
                                          oc.data<T>(), ol.data<I>(), one.data<I>(), n_copies, \
                                          n_features, n_clusters, (int64_t)wgs, q.stream))
    if (dT == DT::F32 && iT == DT::I32) RCD(f32_i32, float, int32_t);
    else if (dT == DT::F32 && iT == DT::I64) RCD(f32_i64, float, int64_t);
    else if (dT == DT::F64 && iT == DT::I32) RCD(f64_i32, double, int32_t);
    else if (dT == DT::F64 && iT == DT::I64) RCD(f64_i64, double, int64_t);
    else throw py::value_error("Unsupported data types");
#undef RCD
    return make_events(q, {szc, cc, osz, oc, ol, one});
}

// _kmeans_lloyd.cpp:284-337
std::pair<Event, Event> py_compute_threshold(py::object d0, size_t topk, py::object t0,
                                             py::object qo, std::vector<Event> depends) {
    Arr data = as_arr(d0), thr = as_arr(t0);
    Queue q = as_queue(qo);
    if (!is_1d(data) || !all_c_contiguous({data, thr}))
        throw py::value_error("Argument data must be a C-contiguous vector");
    if (!is_0d(thr)) throw py::value_error("Argument threshold must be 1-element array");
    if (!same_typenum_as(data.dt, {thr}))
        throw py::value_error("Data types of arguments must be the same");
    if (!queues_are_compatible(q, {data, thr}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    int64_t n = data.get_shape(0);
    if (topk == 0) return {Event(), Event()};
    wait_on(q, depends);
    if (data.dt == DT::F32)
        check(kmc_compute_threshold_f32(data.data<float>(), n, (int64_t)topk, thr.data<float>(),
                                        q.stream));
    else if (data.dt == DT::F64)
        check(kmc_compute_threshold_f64(data.data<double>(), n, (int64_t)topk,
                                        thr.data<double>(), q.stream));
    else
        throw py::value_error(
            "Unsupported elemental data type. Expect single- or double- floating-point types.");
    return make_events(q, {data, thr});
}

// _kmeans_lloyd.cpp:339-441
std::pair<Event, Event> py_select_samples_far_from_centroid(size_t n_selected, py::object a0,
                                                            py::object a1, py::object a2,
                                                            py::object a3, py::object a4,
                                                            size_t wgs, py::object qo,
                                                            std::vector<Event> depends) {
    if (n_selected == 0) throw py::value_error("Argument `n_selected` must be positive");
    Arr dist = as_arr(a0), thr = as_arr(a1), sel = as_arr(a2), ngt = as_arr(a3),
        neq = as_arr(a4);
    Queue q = as_queue(qo);
    if (!is_1d(dist) || !is_1d(sel) || !is_0d(thr) || !is_0d(ngt) || !is_0d(neq))
        throw py::value_error("Array dimensionalities are not consistent");
    int64_t n = dist.get_shape(0);
    if ((size_t)n < n_selected) throw py::value_error("Argument `n_select` is too large");
    if (n != sel.get_shape(0))
        throw py::value_error("Vector `selected_samples_idx` must have size `n_samples`");
    if (!all_c_contiguous({dist, sel})) throw py::value_error("Arrays must be C-contiguous");
    DT dT = dist.dt;
    if (!same_typenum_as(dT, {thr}))
        throw py::value_error("Input arrays must have the same elemental data type");
    DT iT = sel.dt;
    if (!same_typenum_as(iT, {ngt, neq}))
        throw py::value_error("Output array must have the same elemental data type");
    if (!queues_are_compatible(q, {dist, thr, sel, ngt, neq}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    wait_on(q, depends);
#define SEL(SUF, T, I)                                                                        \
    check(kmc_select_samples_far_from_centroid_##SUF((int64_t)n_selected, dist.data<T>(),    \
                                                     thr.data<T>(), sel.data<I>(),           \
                                                     ngt.data<I>(), neq.data<I>(), n,        \
                                                     (int64_t)wgs, q.stream))
    if (dT == DT::F32 && iT == DT::I32) SEL(f32_i32, float, int32_t);
    else if (dT == DT::F64 && iT == DT::I32) SEL(f64_i32, double, int32_t);
    else if (dT == DT::F32 && iT == DT::I64) SEL(f32_i64, float, int64_t);
    else if (dT == DT::F64 && iT == DT::I64) SEL(f64_i64, double, int64_t);
    else throw py::value_error("Unsupported data types");
#undef SEL
    return make_events(q, {dist, thr, sel, ngt, neq});
}

// _kmeans_lloyd.cpp:443-589
std::pair<Event, Event> py_relocate_empty_clusters(size_t n_empty, py::object a0, py::object a1,
                                                   py::object a2, py::object a3, py::object a4,
                                                   py::object a5, py::object a6, py::object a7,
                                                   size_t wgs, py::object qo,
                                                   std::vector<Event> depends) {
    Arr X = as_arr(a0), w = as_arr(a1), lab = as_arr(a2), lst = as_arr(a3), sq = as_arr(a4),
        C = as_arr(a5), sz = as_arr(a6), inr = as_arr(a7);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_1d(w) || !is_1d(lab) || !is_1d(lst) || !is_1d(sq) || !is_2d(C) ||
        !is_1d(sz) || !is_1d(inr))
        throw py::value_error("Arguments have inconsistent array dimensionality.");
    if (!all_c_contiguous({X, w, lab, lst, sq, C, sz, inr}))
        throw py::value_error("Inputs must be C-contiguous");
    int64_t n = X.get_shape(1), d = X.get_shape(0), k = lst.get_shape(0);
    if (n != w.get_shape(0) || n != lab.get_shape(0) || n != sq.get_shape(0) ||
        k != C.get_shape(1) || d != C.get_shape(0) || k != sz.get_shape(0) ||
        n != inr.get_shape(0))
        throw py::value_error("Input dimensions are inconsistent");
    if (n_empty == 0) throw py::value_error("n_empty_clusters must be non-zero.");
    if (!queues_are_compatible(q, {X, w, lab, lst, sq, C, sz, inr}))
        throw py::value_error("Execution queue is not compatible with allocation queues.");
    DT dT = X.dt, iT = lab.dt;
    if (!same_typenum_as(dT, {w, sq, C, sz, inr}) || !same_typenum_as(iT, {lst}))
        throw py::value_error("Inconsistent array elemental data types");
    wait_on(q, depends);
#define REL(SUF, T, I)                                                                        \
    check(kmc_relocate_empty_clusters_##SUF((int64_t)n_empty, X.data<T>(), w.data<T>(),       \
                                            lab.data<I>(), lst.data<I>(), sq.data<T>(),       \
                                            C.data<T>(), sz.data<T>(), inr.data<T>(), n, d, k, \
                                            (int64_t)wgs, q.stream))
    if (dT == DT::F32 && iT == DT::I32) REL(f32_i32, float, int32_t);
    else if (dT == DT::F32 && iT == DT::I64) REL(f32_i64, float, int64_t);
    else if (dT == DT::F64 && iT == DT::I32) REL(f64_i32, double, int32_t);
    else if (dT == DT::F64 && iT == DT::I64) REL(f64_i64, double, int64_t);
    else throw py::value_error("Unsupported data types");
#undef REL
    return make_events(q, {X, w, lab, lst, sq, C, sz, inr});
}

// _kmeans_lloyd.cpp:591-664
std::pair<Event, Event> py_compute_centroid_shifts_squared(py::object a0, py::object a1,
                                                           py::object a2, py::object qo,
                                                           std::vector<Event> depends) {
    Arr oldc = as_arr(a0), newc = as_arr(a1), out = as_arr(a2);
    Queue q = as_queue(qo);
    if (!is_2d(newc) || !is_2d(oldc) || !is_1d(out))
        throw py::value_error("Input dimensionalities are not consistent.");
    int64_t d = oldc.get_shape(0), k = oldc.get_shape(1);
    if (d != newc.get_shape(0) || k != newc.get_shape(1) || k != out.get_shape(0))
        throw py::value_error("Array dimensions are not consistent.");
    if (!all_c_contiguous({newc, oldc, out}))
        throw py::value_error("Arguments must be C-contiguous arrays");
    if (!queues_are_compatible(q, {newc, oldc, out}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    DT t = oldc.dt;
    if (!same_typenum_as(t, {newc, out}))
        throw py::value_error("All array arguments must have the same elemental data types");
    wait_on(q, depends);
    if (t == DT::F32)
        check(kmc_compute_centroid_shifts_squared_f32(oldc.data<float>(), newc.data<float>(),
                                                      out.data<float>(), d, k, q.stream));
    else if (t == DT::F64)
        check(kmc_compute_centroid_shifts_squared_f64(oldc.data<double>(), newc.data<double>(),
                                                      out.data<double>(), d, k, q.stream));
    else
        throw py::value_error("Unsupported elemental data type.");
    return make_events(q, {oldc, newc, out});
}

// _kmeans_lloyd.cpp:666-745
std::pair<Event, Event> py_compute_distances(py::object a0, py::object a1, py::object a2,
                                             size_t wgs, size_t h, py::object qo,
                                             std::vector<Event> depends) {
    Arr X = as_arr(a0), C = as_arr(a1), D = as_arr(a2);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_2d(C) || !is_2d(D))
        throw py::value_error("Input arrays must have dimensionality 2.");
    if (!all_c_contiguous({X, C, D})) throw py::value_error("Input arrays must be C-contiguous.");
    int64_t d = X.get_shape(0), n = X.get_shape(1), k = D.get_shape(0);
    if (d != C.get_shape(0) || k != C.get_shape(1) || n != D.get_shape(1))
        throw py::value_error("Input array dimensions are not consistant");
    if (!queues_are_compatible(q, {X, C, D}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    DT t = X.dt;
    if (!same_typenum_as(t, {C, D}))
        throw py::value_error("Arrays must have the same elemental data types");
    wait_on(q, depends);
    if (t == DT::F32)
        check(kmc_compute_centroid_to_sample_distances_f32(X.data<float>(), C.data<float>(),
                                                           D.data<float>(), n, d, k,
                                                           (int64_t)wgs, (int64_t)h, q.stream));
    else if (t == DT::F64)
        check(kmc_compute_centroid_to_sample_distances_f64(X.data<double>(), C.data<double>(),
                                                           D.data<double>(), n, d, k,
                                                           (int64_t)wgs, (int64_t)h, q.stream));
    else
        throw py::value_error("Unsupported elemental data type");
    return make_events(q, {X, C, D});
}

// _kmeans_lloyd.cpp:747-839
std::pair<Event, Event> py_assignment(py::object a0, py::object a1, py::object a2, py::object a3,
                                      size_t h, size_t wgs, py::object qo,
                                      std::vector<Event> depends) {
    Arr X = as_arr(a0), C = as_arr(a1), hn = as_arr(a2), lab = as_arr(a3);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_2d(C) || !is_1d(hn) || !is_1d(lab))
        throw py::value_error("Inputs have unexpected dimensionality.");
    if (!all_c_contiguous({X, C, hn, lab}))
        throw py::value_error("Inputs must be C-contiguous arrays.");
    int64_t d = X.get_shape(0), n = X.get_shape(1), k = hn.get_shape(0);
    if (d != C.get_shape(0) || k != C.get_shape(1) || n != lab.get_shape(0))
        throw py::value_error("Inputs have inconsistent dimensions.");
    if (!queues_are_compatible(q, {X, C, hn, lab}))
        throw py::value_error("Execution queue is incompatible with allocation queues.");
    DT dT = X.dt, iT = lab.dt;
    if (!same_typenum_as(dT, {C, hn}))
        throw py::value_error("Arrays have inconsistent elemental data types");
    wait_on(q, depends);
#define ASG(SUF, T, I)                                                                        \
    check(kmc_assignment_##SUF(X.data<T>(), C.data<T>(), hn.data<T>(), lab.data<I>(), n, d, k, \
                               (int64_t)h, (int64_t)wgs, q.stream))
    if (dT == DT::F32 && iT == DT::I32) ASG(f32_i32, float, int32_t);
    else if (dT == DT::F64 && iT == DT::I32) ASG(f64_i32, double, int32_t);
    else if (dT == DT::F32 && iT == DT::I64) ASG(f32_i64, float, int64_t);
    else if (dT == DT::F64 && iT == DT::I64) ASG(f64_i64, double, int64_t);
    else throw py::value_error("Unsupported array elemental data type");
#undef ASG
    return make_events(q, {X, C, hn, lab});
}

// _kmeans_lloyd.cpp:841-939
std::pair<Event, Event> py_compute_inertia(py::object a0, py::object a1, py::object a2,
                                           py::object a3, py::object a4, size_t wgs,
                                           py::object qo, std::vector<Event> depends) {
    Arr X = as_arr(a0), w = as_arr(a1), C = as_arr(a2), lab = as_arr(a3), out = as_arr(a4);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_1d(w) || !is_2d(C) || !is_1d(lab) || !is_1d(out))
        throw py::value_error("Input array dimensionality is not consistent");
    if (!all_c_contiguous({X, w, C, lab, out}))
        throw py::value_error("All input arrays must be C-contiguous");
    if (!queues_are_compatible(q, {X, w, C, lab, out}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    int64_t d = X.get_shape(0), n = X.get_shape(1), k = C.get_shape(1);
    if (d != C.get_shape(0) || n != w.get_shape(0) || n != lab.get_shape(0) ||
        n != out.get_shape(0))
        throw py::value_error("Array dimensions are not consistent");
    DT dT = X.dt, iT = lab.dt;
    if (!same_typenum_as(dT, {w, C, out}))
        throw py::value_error("Array elemental data types are not consistent");
    wait_on(q, depends);
#define INR(SUF, T, I)                                                                        \
    check(kmc_compute_inertia_##SUF(X.data<T>(), w.data<T>(), C.data<T>(), lab.data<I>(),     \
                                    out.data<T>(), n, d, k, (int64_t)wgs, q.stream))
    if (dT == DT::F32 && iT == DT::I32) INR(f32_i32, float, int32_t);
    else if (dT == DT::F64 && iT == DT::I32) INR(f64_i32, double, int32_t);
    else if (dT == DT::F32 && iT == DT::I64) INR(f32_i64, float, int64_t);
    else if (dT == DT::F64 && iT == DT::I64) INR(f64_i64, double, int64_t);
    else throw py::value_error("Unsupported array elemental data type");
#undef INR
    return make_events(q, {X, w, C, lab, out});
}

// _kmeans_lloyd.cpp:941-976
py::object py_reduce_vector_blocking(py::object a0, py::object qo, std::vector<Event> depends) {
    Arr data = as_arr(a0);
    Queue q = as_queue(qo);
    if (!is_1d(data) || !all_c_contiguous({data}))
        throw py::value_error("Expecting 1D contiguous vector.");
    if (!queues_are_compatible(q, {data}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    int64_t n = data.get_shape(0);
    wait_on(q, depends);
    if (data.dt == DT::F32) {
        float r = 0.f;
        check(kmc_reduce_vector_blocking_f32(data.data<float>(), n, q.stream, &r));
        return py::cast(r);
    } else if (data.dt == DT::F64) {
        double r = 0.0;
        check(kmc_reduce_vector_blocking_f64(data.data<double>(), n, q.stream, &r));
        return py::cast(r);
    }
    throw py::value_error("Unsupported data type");
}

// _kmeans_lloyd.cpp:980-1109
std::pair<Event, Event> py_fused_lloyd_single_step(py::object a0, py::object a1, py::object a2,
                                                   py::object a3, py::object a4, py::object a5,
                                                   py::object a6, size_t h, size_t wgs,
                                                   py::object qo, std::vector<Event> depends) {
    Arr X = as_arr(a0), w = as_arr(a1), C = as_arr(a2), hn = as_arr(a3), lab = as_arr(a4),
        cc = as_arr(a5), szc = as_arr(a6);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_1d(w) || !is_2d(C) || !is_1d(hn) || !is_1d(lab) || !is_3d(cc) ||
        !is_2d(szc))
        throw py::value_error("Unexpected input array dimensionalities.");
    if (!all_c_contiguous({X, w, C, hn, lab, cc, szc}))
        throw py::value_error("All arrays must be C-contiguous");
    int64_t d = X.get_shape(0), n = X.get_shape(1), k = hn.get_shape(0), P = cc.get_shape(0);
    if (d != C.get_shape(0) || k != C.get_shape(1) || n != w.get_shape(0) ||
        n != lab.get_shape(0) || d != cc.get_shape(1) || k != cc.get_shape(2) ||
        P != szc.get_shape(0) || k != szc.get_shape(1))
        throw py::value_error("Unexpected array dimensions");
    if (!queues_are_compatible(q, {X, w, C, hn, lab, cc, szc}))
        throw py::value_error("Execution queue is not compatible with allocation queues.");
    DT dT = X.dt, iT = lab.dt;
    if (!same_typenum_as(dT, {w, C, hn, cc, szc}))
        throw py::value_error("Array arguments have different elemental data types");
    wait_on(q, depends);
#define FLS(SUF, T, I)                                                                        \
    check(kmc_fused_lloyd_single_step_##SUF(X.data<T>(), w.data<T>(), C.data<T>(),            \
                                            hn.data<T>(), lab.data<I>(), cc.data<T>(),        \
                                            szc.data<T>(), n, d, k, P, (int64_t)h,            \
                                            (int64_t)wgs, q.stream))
    if (dT == DT::F32 && iT == DT::I32) FLS(f32_i32, float, int32_t);
    else if (dT == DT::F32 && iT == DT::I64) FLS(f32_i64, float, int64_t);
    else if (dT == DT::F64 && iT == DT::I32) FLS(f64_i32, double, int32_t);
    else if (dT == DT::F64 && iT == DT::I64) FLS(f64_i64, double, int64_t);
    else throw py::value_error("Unsupported array elemental data types.");
#undef FLS
    return make_events(q, {X, w, C, hn, lab, cc, szc});
}

// _kmeans_lloyd.cpp:1111-1147
size_t py_compute_number_of_private_copies(py::object a0, size_t n, size_t d, size_t k,
                                           double occ, size_t wgs) {
    Arr arr = as_arr(a0);
    if (occ <= 0.0 || occ >= 1.0)
        throw py::value_error("Expecting a fraction strictly between 0 and 1");
    int64_t esize;
    if (arr.dt == DT::F32) esize = 4;
    else if (arr.dt == DT::F64) esize = 8;
    else throw py::value_error("Unsupported elemental data type");
    int64_t out = 0;
    check(kmc_compute_number_of_private_copies(esize, (int64_t)n, (int64_t)d, (int64_t)k, occ,
                                               (int64_t)wgs, 0, &out));
    return (size_t)out;
}

void print_cb(const char *line, void *) { py::print(std::string(line) + "\n"); }

int form_code(const std::string &form) {
    if (form == "plain") return KMC_FORM_PLAIN;
    if (form == "mixed-bf16") return KMC_FORM_MIXED_BF16;
    if (form == "mixed-fp16") return KMC_FORM_MIXED_FP16;
    throw py::value_error("form must be 'plain', 'mixed-fp16' or 'mixed-bf16'");
}

// Mixed tensor-core forms through a fit session (same loop, same results
// contract: init_centroid_t is overwritten, res_centroids_t holds the result).
template <typename I>
int64_t run_mixed_fit(const Arr &X, const Arr &w, const Arr &ic, const Arr &lab, const Arr &rc,
                      int64_t n, int64_t d, int64_t k, double tol, int64_t max_iter, int form,
                      const Queue &q, float *inertia_out) {
    kmc_fit_t fit = nullptr;
    int rc_;
    if (sizeof(I) == 4)
        rc_ = kmc_fit_create_f32_i32(X.data<float>(), w.data<float>(), ic.data<float>(),
                                     lab.data<int32_t>(), rc.data<float>(), n, d, k, tol, max_iter,
                                     form, q.stream, &fit);
    else
        rc_ = kmc_fit_create_f32_i64(X.data<float>(), w.data<float>(), ic.data<float>(),
                                     lab.data<int64_t>(), rc.data<float>(), n, d, k, tol, max_iter,
                                     form, q.stream, &fit);
    check(rc_);
    int64_t it = 0;
    double inr = 0.0;
    int r1 = kmc_fit_run(fit);
    int r2 = (r1 == KMC_OK) ? kmc_fit_finalize(fit, &it, &inr) : r1;
    kmc_fit_destroy(fit);
    check(r2);
    *inertia_out = (float)inr;
    return it;
}

// _kmeans_lloyd.cpp:1149-1275
std::pair<size_t, py::array> py_kmeans_lloyd_driver(py::object a0, py::object a1, py::object a2,
                                                    py::object a3, py::object a4, double tol,
                                                    bool verbose, size_t max_iter, size_t h,
                                                    size_t wgs, double occ, py::object qo,
                                                    std::vector<Event> depends,
                                                    std::string form) {
    Arr X = as_arr(a0), w = as_arr(a1), ic = as_arr(a2), lab = as_arr(a3), rc = as_arr(a4);
    Queue q = as_queue(qo);
    if (!is_2d(X) || !is_1d(w) || !is_2d(ic) || !is_2d(rc) || !is_1d(lab))
        throw py::value_error("Unsupported array dimensionalities");
    if (!all_c_contiguous({X, w, ic, lab, rc}))
        throw py::value_error("All input arrays must be C-contiguous");
    if (!queues_are_compatible(q, {X, w, ic, lab, rc}))
        throw py::value_error("Execution queue is not compatible with allocation queues");
    int64_t d = X.get_shape(0), n = X.get_shape(1), k = ic.get_shape(1);
    if (d != ic.get_shape(0) || d != rc.get_shape(0) || k != rc.get_shape(1) ||
        n != w.get_shape(0) || n != lab.get_shape(0))
        throw py::value_error("Array dimensions are not consistent");
    DT dT = X.dt, iT = lab.dt;
    if (!same_typenum_as(dT, {w, ic, rc}))
        throw py::value_error(
            "Sample coordinates, weights and centroids must have the same elemental data types");
    if (occ <= 0.0 || occ >= 1.0)
        throw py::value_error("Fraction `centroids_private_copies_max_cache_occupancy` is out of bounds");
    if (tol < 0.0) throw py::value_error("Tolerance must be non-negative");
    const int fcode = form_code(form);
    wait_on(q, depends);
    int64_t n_iters = 0;
    py::array res;
    if (fcode != KMC_FORM_PLAIN) {
        if (dT != DT::F32 || (iT != DT::I32 && iT != DT::I64))
            throw py::value_error("mixed forms need float32 data and int32/int64 labels");
        if (verbose) throw py::value_error("verbose output is only available for form='plain'");
        auto tmp = py::array_t<float>(1);
        float *out = tmp.mutable_data(0);
        res = py::cast<py::array>(tmp);
        n_iters = (iT == DT::I32)
                      ? run_mixed_fit<int32_t>(X, w, ic, lab, rc, n, d, k, tol, (int64_t)max_iter,
                                               fcode, q, out)
                      : run_mixed_fit<int64_t>(X, w, ic, lab, rc, n, d, k, tol, (int64_t)max_iter,
                                               fcode, q, out);
        return {(size_t)n_iters, res};
    }
#define DRV(SUF, T, I)                                                                        \
    {                                                                                         \
        auto tmp = py::array_t<T>(1);                                                         \
        T *out = tmp.mutable_data(0);                                                         \
        res = py::cast<py::array>(tmp);                                                       \
        check(kmc_lloyd_driver_##SUF(X.data<T>(), w.data<T>(), ic.data<T>(), lab.data<I>(),   \
                                     rc.data<T>(), n, d, k, tol, verbose ? 1 : 0,             \
                                     (int64_t)max_iter, (int64_t)h, (int64_t)wgs, occ,        \
                                     q.stream, verbose ? print_cb : nullptr, nullptr,         \
                                     &n_iters, out));                                         \
    }
    if (dT == DT::F32 && iT == DT::I32) DRV(f32_i32, float, int32_t)
    else if (dT == DT::F64 && iT == DT::I32) DRV(f64_i32, double, int32_t)
    else if (dT == DT::F32 && iT == DT::I64) DRV(f32_i64, float, int64_t)
    else if (dT == DT::F64 && iT == DT::I64) DRV(f64_i64, double, int64_t)
    else throw py::value_error("Unsupport elemental data type");
#undef DRV
    return {(size_t)n_iters, res};
}

}  // namespace

PYBIND11_MODULE(_kmeans_dpcpp, m) {
    m.doc() = "GB300 (sm_103a) Lloyd k-means engine with the kmeans_dpcpp Python surface.";

    py::class_<Event>(m, "Event")
        .def(py::init<>())
        .def("wait", &Event::wait, "Block until the work recorded by this event completes.")
        .def_property_readonly("is_complete", &Event::is_complete);

    m.def("broadcast_divide", &py_broadcast_divide,
          "broadcast_divide(divident=src, divisor=dst, sycl_queue=q, depends=[]) evaluates "
          "`src /= dst` for matrix src and vector dst",
          py::arg("divident"), py::arg("divisor"), py::arg("work_group_size"),
          py::arg("sycl_queue"), py::arg("depends") = std::vector<Event>());
    m.def("half_l2_norm_squared", &py_half_l2_norm_squared,
          "half_l2_norm_squared(centroids=X, centroids_half_l2_norm_squared=y, sycl_queue=q, "
          "depends=[]) computes row-wise half of norm squared of X and places it in y",
          py::arg("centroids"), py::arg("centroids_half_l2_norm_squared"),
          py::arg("work_group_size"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("reduce_centroids_data", &py_reduce_centroids_data,
          "reduce_centroids_data(cluster_sizes_private_copies, centroids_t_private_copies, "
          "out_cluster_sizes, out_centroids_t, out_empty_clusters_list, out_n_empty_clusters, "
          "sycl_queue=q, depends=[])",
          py::arg("cluster_sizes_private_copies"), py::arg("centroids_t_private_copies"),
          py::arg("out_cluster_sizes"), py::arg("out_centroids_t"),
          py::arg("out_empty_clusters_list"), py::arg("out_n_empty_clusters"),
          py::arg("work_group_size"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("compute_threshold", &py_compute_threshold,
          "compute_threshold(data, topk, threshold, sycl_queue=q, depends=[]) finds topk-th "
          "largest element in data and puts in threshold",
          py::arg("data"), py::arg("topk"), py::arg("threshold"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("select_samples_far_from_centroid", &py_select_samples_far_from_centroid,
          "Populates `selected_samples_idx` with ids of observations whose distance to nearest "
          "centroid is greater than `threshold` (front) or equal to it (back).",
          py::arg("n_selected"), py::arg("distance_to_centroid"), py::arg("threshold"),
          py::arg("selected_samples_idx"), py::arg("n_selected_gt_threshold"),
          py::arg("n_selected_eq_threshold"), py::arg("work_group_size"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("relocate_empty_clusters", &py_relocate_empty_clusters,
          "Relocates empty clustsers, modifies centroid_t, cluster_sizes, per_sample_inertia",
          py::arg("n_empty_clusters"), py::arg("X_t"), py::arg("sample_weights"),
          py::arg("assignment_id"), py::arg("empty_clusters_list"),
          py::arg("sq_dist_to_nearest_centroid"), py::arg("centroid_t"),
          py::arg("cluster_sizes"), py::arg("per_sample_inertia"), py::arg("work_group_size"),
          py::arg("sycl_queue"), py::arg("depends") = std::vector<Event>());
    m.def("compute_centroid_shifts_squared", &py_compute_centroid_shifts_squared,
          "Computes equivalent of `np.sum(np.square(old_centroid_t - new_centroid_t), axis=0)",
          py::arg("centroid_t"), py::arg("new_centroid_t"), py::arg("out_centroid_shifts"),
          py::arg("sycl_queue"), py::arg("depends") = std::vector<Event>());
    m.def("compute_centroid_to_sample_distances", &py_compute_distances,
          "Computes distances from centroids to samples. Inputs: X_t - samples with shape "
          "(n_features, n_samples), centroid_t - centroids with shape (n_features, n_clusters), "
          "and output - euclidean_distances_t with shape (n_clusters, n_samples).",
          py::arg("X_t"), py::arg("centroid_t"), py::arg("euclidean_distances_t"),
          py::arg("work_group_size"), py::arg("centroids_window_height"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("assignment", &py_assignment, "Compute assignment of samples to nearest centroids.",
          py::arg("X_t"), py::arg("centroids_t"), py::arg("centroids_half_l2_norm"),
          py::arg("assignment_id"), py::arg("centroids_window_height"),
          py::arg("work_group_size"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("compute_inertia", &py_compute_inertia,
          "Computes per sample inertia given assignment IDs", py::arg("X_t"),
          py::arg("sample_weight"), py::arg("centroid_t"), py::arg("assignment_id"),
          py::arg("out_per_sample_inertia"), py::arg("work_group_size"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("reduce_vector_blocking", &py_reduce_vector_blocking,
          "Synchronously compute the total value of elements in the vector", py::arg("data"),
          py::arg("sycl_queue"), py::arg("depends") = std::vector<Event>());
    m.def("fused_lloyd_single_step", &py_fused_lloyd_single_step,
          "Perform single step of Lloyd' algorithm for KMeans problem", py::arg("X_t"),
          py::arg("sample_weight"), py::arg("centroids_t"), py::arg("centroids_half_l2_norm"),
          py::arg("assignments_idx"), py::arg("new_centroids_t_private_copies"),
          py::arg("cluster_sizes_private_copies"), py::arg("centroids_window_height"),
          py::arg("work_group_size"), py::arg("sycl_queue"),
          py::arg("depends") = std::vector<Event>());
    m.def("compute_number_of_private_copies", &py_compute_number_of_private_copies,
          "Computes optimal number of private copies parametrized by max-cache-ocupancy fraction.",
          py::arg("array"), py::arg("n_samples"), py::arg("n_features"), py::arg("n_clusters"),
          py::arg("centroids_private_copies_max_cache_occupancy"), py::arg("work_group_size"));
    m.def("kmeans_lloyd_driver", &py_kmeans_lloyd_driver,
          "Implement Lloyd's refinement algorithm. Returns 2-tuple, number of iterations "
          "performed and 0d numpy array with total_inertia of the returned configuration. "
          "Array init_centroid_t is overwritten.",
          py::arg("X_t"), py::arg("sample_weight"), py::arg("init_centroid_t"),
          py::arg("assignments_id"), py::arg("res_centroids_t"), py::arg("tol"),
          py::arg("verbose"), py::arg("max_iter"), py::arg("centroids_window_height"),
          py::arg("work_group_size"), py::arg("centroids_private_copies_max_cache_occupancy"),
          py::arg("sycl_queue"), py::arg("depends") = std::vector<Event>(),
          py::arg("form") = std::string("plain"));
}
