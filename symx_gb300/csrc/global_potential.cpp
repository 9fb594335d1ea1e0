#include "global_potential.h"

#include <cstring>
#include <stdexcept>

namespace symx {

ConnectivityMap GlobalPotential::flat_connectivity(const std::vector<int32_t>& conn, int32_t stride)
{
    if (stride <= 0 || conn.size() % (size_t)stride != 0)
        throw std::runtime_error("symx: connectivity size is not a multiple of its stride");
    const std::vector<int32_t>* c = &conn;
    ConnectivityMap m;
    m.data = [c]() { return c->data(); };
    m.n_elements = [c, stride]() { return (int64_t)c->size() / stride; };
    m.stride = stride;
    return m;
}

void GlobalPotential::add_potential(const std::string& name, const ConnectivityMap& conn, const DefFunc& f,
                                    int /*labels_from*/, const std::vector<std::string>& labels)
{
    auto mws = std::make_shared<MappedWorkspace<double>>(conn);
    mws->set_name(name);
    Element e(conn.stride);
    e.set_labels(labels);
    Potential p;
    p.name = name;
    p.mws = mws;
    p.expression = f(*mws, e);
    if (p.expression.graph != mws->ws.graph.get())
        throw std::runtime_error("symx: potential '" + name + "' returned an expression of another workspace");
    potentials.push_back(p);
}

void GlobalPotential::add_potential(const std::string& name, const ConnectivityMap& conn, const DefFuncConditional& f,
                                    const std::vector<std::string>& labels)
{
    auto mws = std::make_shared<MappedWorkspace<double>>(conn);
    mws->set_name(name);
    Element e(conn.stride);
    e.set_labels(labels);
    Potential p;
    p.name = name;
    p.mws = mws;
    auto pc = f(*mws, e);
    p.expression = pc.first;
    p.condition = pc.second;
    p.has_condition = true;
    potentials.push_back(p);
}

void GlobalPotential::add_dof_raw(std::uintptr_t id, std::function<double*()> data, std::function<int64_t()> n_dofs)
{
    for (const DofSet& d : dofs)
        if (d.id == id) throw std::runtime_error("symx: DoF array registered twice");
    DofSet d;
    d.id = id;
    d.data = std::move(data);
    d.n_dofs = std::move(n_dofs);
    if (d.n_dofs() % 3 != 0) throw std::runtime_error("symx: DoF arrays must have 3 values per item");
    dofs.push_back(d);
}

int GlobalPotential::get_total_n_dofs() const
{
    int64_t n = 0;
    for (const DofSet& d : dofs) n += d.n_dofs();
    return (int)n;
}

std::vector<int> GlobalPotential::get_dofs_offsets() const
{
    std::vector<int> off{0};
    for (const DofSet& d : dofs) off.push_back(off.back() + (int)d.n_dofs());
    return off;
}

void GlobalPotential::get_dofs(double* out) const
{
    int64_t o = 0;
    for (const DofSet& d : dofs) {
        const int64_t n = d.n_dofs();
        std::memcpy(out + o, d.data(), sizeof(double) * n);
        o += n;
    }
}

void GlobalPotential::set_dofs(const double* in)
{
    int64_t o = 0;
    for (const DofSet& d : dofs) {
        const int64_t n = d.n_dofs();
        std::memcpy(d.data(), in + o, sizeof(double) * n);
        o += n;
    }
}

void GlobalPotential::apply_dof_increment(const double* du)
{
    int64_t o = 0;
    for (const DofSet& d : dofs) {
        const int64_t n = d.n_dofs();
        double* x = d.data();
        for (int64_t i = 0; i < n; ++i) x[i] += du[o + i];
        o += n;
    }
}

}  // namespace symx
