// Global potential = sum of element potentials over connectivities + the degrees of
// freedom they are minimised over (reference: symx/src/solver/{GlobalPotential,Potential}.h).
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "mapped_workspace.h"

namespace symx {

using DefFunc = std::function<Scalar(MappedWorkspace<double>&, Element&)>;
// A potential with an activity condition: the element contributes only where cond > 0.
using DefFuncConditional = std::function<std::pair<Scalar, Scalar>(MappedWorkspace<double>&, Element&)>;

struct Potential {
    std::string name;
    std::shared_ptr<MappedWorkspace<double>> mws;
    Scalar expression;
    bool has_condition = false;
    Scalar condition;
};

// A flat array of degrees of freedom owned by the user (3 per vertex).
struct DofSet {
    std::uintptr_t id = 0;
    std::function<double*()> data;
    std::function<int64_t()> n_dofs;
};

class GlobalPotential {
public:
    static std::shared_ptr<GlobalPotential> create() { return std::make_shared<GlobalPotential>(); }

    void add_potential(const std::string& name, const ConnectivityMap& conn, const DefFunc& f, int labels_from = -1,
                       const std::vector<std::string>& labels = {});
    void add_potential(const std::string& name, const ConnectivityMap& conn, const DefFuncConditional& f,
                       const std::vector<std::string>& labels = {});

    void add_potential(const std::string& name, const std::vector<int32_t>& conn, int32_t stride, const DefFunc& f)
    {
        add_potential(name, flat_connectivity(conn, stride), f);
    }
    void add_potential(const std::string& name, const std::vector<int32_t>& conn, int32_t stride,
                       const DefFuncConditional& f)
    {
        add_potential(name, flat_connectivity(conn, stride), f);
    }
    template <std::size_t N>
    void add_potential(const std::string& name, const std::vector<std::array<int32_t, N>>& conn, const DefFunc& f)
    {
        add_potential(name, array_connectivity(conn), f);
    }
    template <std::size_t N>
    void add_potential(const std::string& name, const std::vector<std::array<int32_t, N>>& conn,
                       const DefFuncConditional& f)
    {
        add_potential(name, array_connectivity(conn), f);
    }
    template <std::size_t N>
    void add_potential(const std::string& name, const LabelledConnectivity<N>& conn, const DefFunc& f)
    {
        add_potential(name, array_connectivity(conn.data), f, 0,
                      std::vector<std::string>(conn.labels.begin(), conn.labels.end()));
    }
    template <std::size_t N>
    void add_potential(const std::string& name, const LabelledConnectivity<N>& conn, const DefFuncConditional& f)
    {
        add_potential(name, array_connectivity(conn.data), f,
                      std::vector<std::string>(conn.labels.begin(), conn.labels.end()));
    }

    // Register a DoF array: std::vector of 3-vectors (Eigen::Vector3d, std::array<double,3>)
    // or a flat std::vector<double> whose size is a multiple of 3.
    template <typename STATIC_VECTOR>
    void add_dof(std::vector<STATIC_VECTOR>& arr)
    {
        static_assert(sizeof(STATIC_VECTOR) % sizeof(double) == 0, "DoF items must be made of doubles");
        std::vector<STATIC_VECTOR>* c = &arr;
        constexpr int64_t per = sizeof(STATIC_VECTOR) / sizeof(double);
        add_dof_raw(reinterpret_cast<std::uintptr_t>(c), [c]() { return reinterpret_cast<double*>(c->data()); },
                    [c]() { return (int64_t)c->size() * per; });
    }
    void add_dof_raw(std::uintptr_t id, std::function<double*()> data, std::function<int64_t()> n_dofs);

    int get_total_n_dofs() const;
    std::vector<int> get_dofs_offsets() const;
    void get_dofs(double* out) const;
    void set_dofs(const double* in);
    void apply_dof_increment(const double* du);
    int get_n_potentials() const { return (int)potentials.size(); }

    std::vector<Potential> potentials;
    std::vector<DofSet> dofs;

private:
    static ConnectivityMap flat_connectivity(const std::vector<int32_t>& conn, int32_t stride);
    template <std::size_t N>
    static ConnectivityMap array_connectivity(const std::vector<std::array<int32_t, N>>& conn)
    {
        const std::vector<std::array<int32_t, N>>* c = &conn;
        ConnectivityMap m;
        m.data = [c]() { return reinterpret_cast<const int32_t*>(c->data()); };
        m.n_elements = [c]() { return (int64_t)c->size(); };
        m.stride = (int32_t)N;
        return m;
    }
};
using spGlobalPotential = std::shared_ptr<GlobalPotential>;

}  // namespace symx
