// Binding of symbols to user data, with the reference's user API
// (symx/src/compile/{MappedWorkspace.h,Element.h,LabelledConnectivity.h,data_maps.h}).
//
// Inside a potential definition the user calls make_scalar/make_vector(s)/make_matrix on
// arrays they own; each call creates symbols and records a DataMap: where the values
// come from (a pointer getter, so data that moves or changes between solves is re-read),
// how many doubles one item has (stride), and which connectivity column selects the item
// (-1 for data shared by all elements).  The code generator turns these maps into the
// per-element gather at the top of each element kernel.
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "symbolic.h"

namespace symx {

struct Index {
    int idx;
};

// Element-local view of one connectivity row: element[i] is column i.
struct Element {
    explicit Element(int n_items) : n(n_items) {}
    Index operator[](int i) const
    {
        if (i < 0 || i >= n) throw std::runtime_error("symx: Element index out of range");
        return Index{i};
    }
    Index operator[](const std::string& label) const
    {
        for (size_t i = 0; i < labels.size(); ++i)
            if (labels[i] == label) return Index{(int)i};
        throw std::runtime_error("symx: Element label not found: " + label);
    }
    std::vector<Index> slice(int begin, int end) const
    {
        std::vector<Index> v;
        for (int i = begin; i < end; ++i) v.push_back((*this)[i]);
        return v;
    }
    std::vector<Index> all() const { return slice(0, n); }
    void set_labels(const std::vector<std::string>& l) { labels = l; }
    int size() const { return n; }

    int n;
    std::vector<std::string> labels;
};

template <std::size_t N>
struct LabelledConnectivity {
    std::array<std::string, N> labels;
    std::vector<std::array<int32_t, N>> data;

    explicit LabelledConnectivity(const std::array<std::string, N>& l) : labels(l) {}
    Element get_element() const
    {
        Element e((int)N);
        e.set_labels(std::vector<std::string>(labels.begin(), labels.end()));
        return e;
    }
    std::array<int32_t, N>& operator[](int i) { return data[i]; }
    const std::array<int32_t, N>& operator[](int i) const { return data[i]; }
    void push_back(const std::array<int32_t, N>& v) { data.push_back(v); }
    void clear() { data.clear(); }
    std::size_t size() const { return data.size(); }
    // Append a row whose column 0 is the row's own number.
    int32_t numbered_push_back(const std::array<int32_t, N - 1>& v)
    {
        std::array<int32_t, N> r;
        r[0] = (int32_t)data.size();
        for (std::size_t i = 0; i + 1 < N; ++i) r[i + 1] = v[i];
        data.push_back(r);
        return r[0];
    }
};

// Where the values of a run of symbols come from.
struct DataMap {
    std::uintptr_t id = 0;                    // identity of the user container (address)
    std::function<const double*()> data;      // current data pointer
    std::function<int64_t()> n_items;         // rows available (-1: global data)
    int32_t stride = 0;                       // doubles per item, = number of symbols bound
    int32_t conn_column = -1;                 // connectivity column selecting the item; -1 = global
    int32_t first_symbol = 0;                 // symbol index of the first value
};

// The connectivity a potential iterates over.
struct ConnectivityMap {
    std::function<const int32_t*()> data;
    std::function<int64_t()> n_elements;
    int32_t stride = 0;
};

// Values substituted into designated symbols once per iteration of a summation (e.g. the
// quadrature points of an FEM rule); the element kernel accumulates all outputs over them.
struct Summation {
    std::vector<double> data;  // n_iterations x stride
    int32_t n_iterations = 0;
    int32_t stride = 0;
    int32_t first_symbol = -1;
};

namespace detail {
template <typename T>
inline std::uintptr_t addr(const T& x) { return reinterpret_cast<std::uintptr_t>(&x); }
// Number of doubles in one fixed-size item (std::array<double,N>, Eigen fixed vectors, ...).
template <typename SV>
constexpr int32_t item_doubles() { return (int32_t)(sizeof(SV) / sizeof(double)); }
}  // namespace detail

template <typename FLOAT = double>
class MappedWorkspace {
    static_assert(std::is_same<FLOAT, double>::value, "symx_gb300: data is bound as double");

public:
    Workspace ws;
    std::vector<DataMap> maps;
    ConnectivityMap conn;
    Summation summation;
    std::string name = "NO_NAME";

    explicit MappedWorkspace(const ConnectivityMap& c) : conn(c) {}

    // ---- data shared by all elements
    Scalar make_scalar(const FLOAT& value)
    {
        const FLOAT* p = &value;
        return bind(detail::addr(value), [p]() { return p; }, [] { return (int64_t)-1; }, 1, -1)[0];
    }
    template <typename STATIC_VECTOR>
    Vector make_vector(const STATIC_VECTOR& arr)
    {
        const FLOAT* p = reinterpret_cast<const FLOAT*>(&arr);
        return Vector(bind(detail::addr(arr), [p]() { return p; }, [] { return (int64_t)-1; },
                           detail::item_doubles<STATIC_VECTOR>(), -1));
    }
    template <typename DYNAMIC_VECTOR>
    Matrix make_matrix(const DYNAMIC_VECTOR& arr, const std::array<int, 2> shape)
    {
        const DYNAMIC_VECTOR* c = &arr;
        return Matrix(bind(detail::addr(arr), [c]() { return (const FLOAT*)c->data(); }, [] { return (int64_t)-1; },
                           shape[0] * shape[1], -1),
                      {shape[0], shape[1]});
    }

    // ---- per-item data selected by a connectivity column
    template <typename DYNAMIC_VECTOR>
    Scalar make_scalar(const DYNAMIC_VECTOR& arr, const Index& idx)
    {
        const DYNAMIC_VECTOR* c = &arr;
        return bind(detail::addr(arr), [c]() { return (const FLOAT*)c->data(); },
                    [c]() { return (int64_t)c->size(); }, 1, idx.idx)[0];
    }
    template <typename DYNAMIC_VECTOR>
    std::vector<Scalar> make_scalars(const DYNAMIC_VECTOR& arr, const std::vector<Index>& indices)
    {
        std::vector<Scalar> out;
        for (const Index& i : indices) out.push_back(make_scalar(arr, i));
        return out;
    }
    template <typename STATIC_VECTOR>
    Vector make_vector(const std::vector<STATIC_VECTOR>& arr, const Index& idx)
    {
        const std::vector<STATIC_VECTOR>* c = &arr;
        return Vector(bind(detail::addr(arr), [c]() { return reinterpret_cast<const FLOAT*>(c->data()); },
                           [c]() { return (int64_t)c->size(); }, detail::item_doubles<STATIC_VECTOR>(), idx.idx));
    }
    template <typename DYNAMIC_VECTOR>
    Vector make_vector(const DYNAMIC_VECTOR& arr, const int32_t stride, const Index& idx)
    {
        const DYNAMIC_VECTOR* c = &arr;
        return Vector(bind(detail::addr(arr), [c]() { return (const FLOAT*)c->data(); },
                           [c, stride]() { return (int64_t)c->size() / stride; }, stride, idx.idx));
    }
    template <typename STATIC_VECTOR>
    std::vector<Vector> make_vectors(const std::vector<STATIC_VECTOR>& arr, const std::vector<Index>& indices)
    {
        std::vector<Vector> out;
        for (const Index& i : indices) out.push_back(make_vector(arr, i));
        return out;
    }
    template <typename STATIC_VECTOR>
    std::vector<Vector> make_vectors(const std::vector<STATIC_VECTOR>& arr, const Element& element)
    {
        return make_vectors(arr, element.all());
    }
    template <typename DYNAMIC_VECTOR>
    std::vector<Vector> make_vectors(const DYNAMIC_VECTOR& arr, const int32_t stride, const std::vector<Index>& indices)
    {
        std::vector<Vector> out;
        for (const Index& i : indices) out.push_back(make_vector(arr, stride, i));
        return out;
    }
    template <typename STATIC_VECTOR>
    Matrix make_matrix(const std::vector<STATIC_VECTOR>& arr, const std::array<int, 2> shape, const Index& idx)
    {
        const std::vector<STATIC_VECTOR>* c = &arr;
        if (detail::item_doubles<STATIC_VECTOR>() != shape[0] * shape[1])
            throw std::runtime_error("symx: make_matrix item size does not match the shape");
        return Matrix(bind(detail::addr(arr), [c]() { return reinterpret_cast<const FLOAT*>(c->data()); },
                           [c]() { return (int64_t)c->size(); }, shape[0] * shape[1], idx.idx),
                      {shape[0], shape[1]});
    }

    // ---- summation over fixed iteration data (e.g. quadrature points)
    template <typename STATIC_VECTOR>
    Scalar add_for_each(const std::vector<STATIC_VECTOR>& iteration_vectors, std::function<Scalar(Vector&)> f)
    {
        if (summation.n_iterations > 0) throw std::runtime_error("symx: one summation per potential");
        const int32_t stride = detail::item_doubles<STATIC_VECTOR>();
        summation.stride = stride;
        summation.n_iterations = (int32_t)iteration_vectors.size();
        summation.first_symbol = ws.get_n_symbols();
        const double* p = reinterpret_cast<const double*>(iteration_vectors.data());
        summation.data.assign(p, p + (size_t)stride * iteration_vectors.size());
        Vector v = ws.make_vector(stride);
        return f(v);
    }
    bool has_summation() const { return summation.n_iterations > 0; }

    Scalar make_zero() { return ws.get_zero(); }
    Scalar make_one() { return ws.get_one(); }
    Vector make_zero_vector(int32_t n) { return ws.get_zero_vector(n); }
    Matrix make_zero_matrix(const std::array<int32_t, 2> shape) { return ws.get_zero_matrix(shape); }
    Matrix make_identity_matrix(int32_t n) { return ws.get_identity_matrix(n); }
    void set_name(const std::string& n) { name = n; }

    int64_t get_n_elements() const { return conn.n_elements(); }
    int32_t get_connectivity_stride() const { return conn.stride; }
    const int32_t* get_connectivity_data() const { return conn.data(); }

    // Checks that every per-item map can be indexed by every element (the reference's
    // verify_no_out_of_bounds, MappedWorkspace.h:658-798).
    void verify_no_out_of_bounds() const
    {
        const int64_t ne = conn.n_elements();
        const int32_t* c = conn.data();
        for (const DataMap& m : maps) {
            if (m.conn_column < 0) continue;
            const int64_t n_items = m.n_items();
            for (int64_t e = 0; e < ne; ++e) {
                const int32_t i = c[e * conn.stride + m.conn_column];
                if (i < 0 || i >= n_items)
                    throw std::runtime_error("symx: potential '" + name + "' indexes item " + std::to_string(i) +
                                             " of an array with " + std::to_string(n_items) + " items");
            }
        }
    }

private:
    std::vector<Scalar> bind(std::uintptr_t id, std::function<const double*()> data, std::function<int64_t()> n_items,
                             int32_t stride, int32_t conn_column)
    {
        if (conn_column >= conn.stride) throw std::runtime_error("symx: connectivity column out of range");
        DataMap m;
        m.id = id;
        m.data = std::move(data);
        m.n_items = std::move(n_items);
        m.stride = stride;
        m.conn_column = conn_column;
        m.first_symbol = ws.get_n_symbols();
        std::vector<Scalar> s = ws.make_scalars(stride);
        maps.push_back(m);
        return s;
    }
};

}  // namespace symx
