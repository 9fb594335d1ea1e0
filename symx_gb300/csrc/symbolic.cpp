// Symbolic front end: DAG construction with local simplification, evaluation,
// hashing and differentiation.  See symbolic.h.
#include "symbolic.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>

namespace symx {

namespace {
uint64_t dbits(double v)
{
    uint64_t u;
    std::memcpy(&u, &v, sizeof(u));
    return u;
}
bool is_commutative(Op op) { return op == Op::Add || op == Op::Mul; }
}  // namespace

size_t Expressions::KeyHash::operator()(const Key& k) const
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t x) { h ^= x; h *= 1099511628211ull; };
    mix((uint64_t)(uint32_t)k.op);
    mix((uint64_t)(uint32_t)k.a);
    mix((uint64_t)(uint32_t)k.b);
    mix((uint64_t)(uint32_t)k.c);
    mix(k.v);
    return (size_t)h;
}

Expressions::Expressions()
{
    nodes_.push_back(Node{Op::Zero, -1, -1, -1, 0.0});
    nodes_.push_back(Node{Op::One, -1, -1, -1, 1.0});
}

int32_t Expressions::constant(double v)
{
    if (v == 0.0 && !std::signbit(v)) return 0;
    if (v == 1.0) return 1;
    return add(Op::Const, -1, -1, -1, v);
}

int32_t Expressions::new_symbol()
{
    Node n{Op::Symbol, -1, -1, -1, (double)n_symbols_};
    nodes_.push_back(n);
    const int32_t id = (int32_t)nodes_.size() - 1;
    symbol_nodes_.push_back(id);
    symbol_values_.push_back(0.0);
    ++n_symbols_;
    return id;
}

void Expressions::set_symbol_value(int32_t symbol_idx, double v) { symbol_values_.at(symbol_idx) = v; }

int32_t Expressions::add(Op op, int32_t a, int32_t b, int32_t c, double v)
{
    auto is_const = [&](int32_t i) {
        const Op o = nodes_[i].op;
        return o == Op::Zero || o == Op::One || o == Op::Const;
    };
    auto cv = [&](int32_t i) { return nodes_[i].v; };
    switch (op) {
        case Op::Add:
            if (a == 0) return b;
            if (b == 0) return a;
            if (is_const(a) && is_const(b)) return constant(cv(a) + cv(b));
            if (nodes_[b].op == Op::Neg) return add(Op::Sub, a, nodes_[b].a);
            if (nodes_[a].op == Op::Neg) return add(Op::Sub, b, nodes_[a].a);
            break;
        case Op::Sub:
            if (b == 0) return a;
            if (a == b) return 0;
            if (is_const(a) && is_const(b)) return constant(cv(a) - cv(b));
            if (a == 0) return add(Op::Neg, b);
            break;
        case Op::Mul:
            if (a == 0 || b == 0) return 0;
            if (a == 1) return b;
            if (b == 1) return a;
            if (is_const(a) && is_const(b)) return constant(cv(a) * cv(b));
            if (is_const(a) && cv(a) == -1.0) return add(Op::Neg, b);
            if (is_const(b) && cv(b) == -1.0) return add(Op::Neg, a);
            break;
        case Op::Div:
            if (b == 1) return a;
            if (a == 0) return 0;
            if (is_const(a) && is_const(b)) return constant(cv(a) / cv(b));
            // a / b with a non-constant denominator becomes a * (1 / b): every quotient by the
            // same b then shares one reciprocal (divisions are the costliest FP64 operation).
            if (!is_const(b) && a != 1) return add(Op::Mul, a, add(Op::Div, 1, b));
            break;
        case Op::Neg:
            if (a == 0) return 0;
            if (is_const(a)) return constant(-cv(a));
            if (nodes_[a].op == Op::Neg) return nodes_[a].a;
            break;
        case Op::PowN:
            if (b == 0) return 1;
            if (b == 1) return a;
            if (a == 1) return 1;
            if (a == 0 && b > 0) return 0;
            if (is_const(a)) return constant(std::pow(cv(a), (double)b));
            break;
        case Op::PowF:
            if (v == 1.0) return a;
            if (v == 0.0) return 1;
            if (is_const(a)) return constant(std::pow(cv(a), v));
            break;
        case Op::Sqrt:
        case Op::Ln:
        case Op::Log10:
        case Op::Exp:
        case Op::Sin:
        case Op::Cos:
        case Op::Tan:
        case Op::Asin:
        case Op::Acos:
        case Op::Atan:
            if (is_const(a)) {
                const double x = cv(a);
                double r = 0.0;
                switch (op) {
                    case Op::Sqrt: r = std::sqrt(x); break;
                    case Op::Ln: r = x <= 0.0 ? -std::numeric_limits<double>::infinity() : std::log(x); break;
                    case Op::Log10: r = x <= 0.0 ? -std::numeric_limits<double>::infinity() : std::log10(x); break;
                    case Op::Exp: r = std::exp(x); break;
                    case Op::Sin: r = std::sin(x); break;
                    case Op::Cos: r = std::cos(x); break;
                    case Op::Tan: r = std::tan(x); break;
                    case Op::Asin: r = std::asin(x); break;
                    case Op::Acos: r = std::acos(x); break;
                    default: r = std::atan(x); break;
                }
                return constant(r);
            }
            break;
        case Op::Branch:
            if (a == b) return a;
            if (is_const(c)) return cv(c) > 0.0 ? a : b;
            break;
        default:
            break;
    }
    if (is_commutative(op) && a > b) std::swap(a, b);
    Key k{(int32_t)op, a, b, c, (op == Op::Const || op == Op::PowF) ? dbits(v) : 0};
    auto it = map_.find(k);
    if (it != map_.end()) return it->second;
    nodes_.push_back(Node{op, a, b, c, v});
    const int32_t id = (int32_t)nodes_.size() - 1;
    map_.emplace(k, id);
    return id;
}

double Expressions::eval(int32_t root) const
{
    std::vector<double> val(root + 1, 0.0);
    for (int32_t i = 0; i <= root; ++i) {
        const Node& n = nodes_[i];
        const double a = n.a >= 0 && n.op != Op::Symbol ? val[n.a] : 0.0;
        const double b = (n.b >= 0 && n.op != Op::PowN) ? val[n.b] : 0.0;
        switch (n.op) {
            case Op::Zero: val[i] = 0.0; break;
            case Op::One: val[i] = 1.0; break;
            case Op::Const: val[i] = n.v; break;
            case Op::Symbol: val[i] = symbol_values_[(int32_t)n.v]; break;
            case Op::Add: val[i] = a + b; break;
            case Op::Sub: val[i] = a - b; break;
            case Op::Mul: val[i] = a * b; break;
            case Op::Div: val[i] = a / b; break;
            case Op::Neg: val[i] = -a; break;
            case Op::PowN: val[i] = std::pow(a, (double)n.b); break;
            case Op::PowF: val[i] = std::pow(a, n.v); break;
            case Op::Sqrt: val[i] = std::sqrt(a); break;
            case Op::Ln: val[i] = a <= 0.0 ? -std::numeric_limits<double>::infinity() : std::log(a); break;
            case Op::Log10: val[i] = a <= 0.0 ? -std::numeric_limits<double>::infinity() : std::log10(a); break;
            case Op::Exp: val[i] = std::exp(a); break;
            case Op::Sin: val[i] = std::sin(a); break;
            case Op::Cos: val[i] = std::cos(a); break;
            case Op::Tan: val[i] = std::tan(a); break;
            case Op::Asin: val[i] = std::asin(a); break;
            case Op::Acos: val[i] = std::acos(a); break;
            case Op::Atan: val[i] = std::atan(a); break;
            case Op::Branch: val[i] = val[n.c] > 0.0 ? a : b; break;
        }
    }
    return val[root];
}

uint64_t Expressions::hash(const std::vector<int32_t>& roots) const
{
    int32_t top = 0;
    for (int32_t r : roots) top = std::max(top, r);
    std::vector<uint8_t> need(top + 1, 0);
    for (int32_t r : roots) need[r] = 1;
    for (int32_t i = top; i >= 0; --i) {
        if (!need[i]) continue;
        const Node& n = nodes_[i];
        if (n.op == Op::Symbol || n.op == Op::Const || n.op == Op::Zero || n.op == Op::One) continue;
        if (n.a >= 0) need[n.a] = 1;
        if (n.b >= 0 && n.op != Op::PowN) need[n.b] = 1;
        if (n.c >= 0) need[n.c] = 1;
    }
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t x) {
        for (int k = 0; k < 8; ++k) { h ^= (x >> (8 * k)) & 0xff; h *= 1099511628211ull; }
    };
    for (int32_t i = 0; i <= top; ++i) {
        if (!need[i]) continue;
        const Node& n = nodes_[i];
        mix((uint64_t)i);
        mix((uint64_t)(uint32_t)n.op);
        mix((uint64_t)(uint32_t)n.a);
        mix((uint64_t)(uint32_t)n.b);
        mix((uint64_t)(uint32_t)n.c);
        mix(dbits(n.v));
    }
    for (int32_t r : roots) mix((uint64_t)(uint32_t)r);
    return h;
}

// ------------------------------------------------------------------ Scalar
namespace {
Scalar mk(const Scalar& ref, Op op, int32_t a, int32_t b = -1, int32_t c = -1, double v = 0.0)
{
    return Scalar(ref.graph->add(op, a, b, c, v), ref.graph);
}
void same_graph(const Scalar& a, const Scalar& b)
{
    if (a.graph != b.graph) throw std::runtime_error("symx: scalars from different workspaces");
}
}  // namespace

bool Scalar::is_constant() const
{
    const Op o = (*graph)[expr_id].op;
    return o == Op::Zero || o == Op::One || o == Op::Const;
}
std::string Scalar::get_checksum() const
{
    char buf[17];
    std::snprintf(buf, sizeof(buf), "%016llx", (unsigned long long)graph->hash({expr_id}));
    return buf;
}

void Scalar::set_value(double v) const
{
    if (!is_symbol()) throw std::runtime_error("symx: set_value on a non-symbol");
    graph->set_symbol_value(get_symbol_idx(), v);
}
Scalar Scalar::operator+(const Scalar& o) const { same_graph(*this, o); return mk(*this, Op::Add, expr_id, o.expr_id); }
Scalar Scalar::operator-(const Scalar& o) const { same_graph(*this, o); return mk(*this, Op::Sub, expr_id, o.expr_id); }
Scalar Scalar::operator*(const Scalar& o) const { same_graph(*this, o); return mk(*this, Op::Mul, expr_id, o.expr_id); }
Scalar Scalar::operator/(const Scalar& o) const { same_graph(*this, o); return mk(*this, Op::Div, expr_id, o.expr_id); }
Scalar Scalar::operator+(double v) const { return *this + make_constant(v); }
Scalar Scalar::operator-(double v) const { return *this - make_constant(v); }
Scalar Scalar::operator*(double v) const { return *this * make_constant(v); }
Scalar Scalar::operator/(double v) const { return *this / make_constant(v); }
Scalar Scalar::powN(int32_t n) const
{
    if (n < 0) return get_one() / powN(-n);
    return mk(*this, Op::PowN, expr_id, n);
}
Scalar Scalar::powF(double p) const { return mk(*this, Op::PowF, expr_id, -1, -1, p); }
Scalar Scalar::inv() const { return get_one() / *this; }
Scalar Scalar::sqrt() const { return mk(*this, Op::Sqrt, expr_id); }
Scalar Scalar::ln() const { return mk(*this, Op::Ln, expr_id); }
Scalar Scalar::log10() const { return mk(*this, Op::Log10, expr_id); }
Scalar Scalar::exp() const { return mk(*this, Op::Exp, expr_id); }
Scalar Scalar::sin() const { return mk(*this, Op::Sin, expr_id); }
Scalar Scalar::cos() const { return mk(*this, Op::Cos, expr_id); }
Scalar Scalar::tan() const { return mk(*this, Op::Tan, expr_id); }
Scalar Scalar::asin() const { return mk(*this, Op::Asin, expr_id); }
Scalar Scalar::acos() const { return mk(*this, Op::Acos, expr_id); }
Scalar Scalar::atan() const { return mk(*this, Op::Atan, expr_id); }

Scalar operator+(double v, const Scalar& s) { return s.make_constant(v) + s; }
Scalar operator-(double v, const Scalar& s) { return s.make_constant(v) - s; }
Scalar operator*(double v, const Scalar& s) { return s.make_constant(v) * s; }
Scalar operator/(double v, const Scalar& s) { return s.make_constant(v) / s; }
Scalar operator-(const Scalar& s) { return mk(s, Op::Neg, s.expr_id); }
Scalar powN(const Scalar& s, int32_t n) { return s.powN(n); }
Scalar powF(const Scalar& s, double p) { return s.powF(p); }
Scalar sqrt(const Scalar& s) { return s.sqrt(); }
Scalar log(const Scalar& s) { return s.ln(); }
Scalar ln(const Scalar& s) { return s.ln(); }
Scalar log10(const Scalar& s) { return s.log10(); }
Scalar exp(const Scalar& s) { return s.exp(); }
Scalar sin(const Scalar& s) { return s.sin(); }
Scalar cos(const Scalar& s) { return s.cos(); }
Scalar tan(const Scalar& s) { return s.tan(); }
Scalar asin(const Scalar& s) { return s.asin(); }
Scalar acos(const Scalar& s) { return s.acos(); }
Scalar atan(const Scalar& s) { return s.atan(); }
Scalar branch(const Scalar& cond, const Scalar& pos, const Scalar& neg)
{
    same_graph(cond, pos);
    same_graph(cond, neg);
    return mk(cond, Op::Branch, pos.expr_id, neg.expr_id, cond.expr_id);
}
Scalar branch(const Scalar& cond, double pos, const Scalar& neg) { return branch(cond, cond.make_constant(pos), neg); }
Scalar branch(const Scalar& cond, const Scalar& pos, double neg) { return branch(cond, pos, cond.make_constant(neg)); }
Scalar branch(const Scalar& cond, double pos, double neg)
{
    return branch(cond, cond.make_constant(pos), cond.make_constant(neg));
}
Scalar operator>(const Scalar& a, const Scalar& b) { return a - b; }
Scalar operator<(const Scalar& a, const Scalar& b) { return b - a; }
Scalar operator>(const Scalar& a, double b) { return a - b; }
Scalar operator<(const Scalar& a, double b) { return b - a; }
Scalar operator>(double a, const Scalar& b) { return a - b; }
Scalar operator<(double a, const Scalar& b) { return b - a; }
Scalar min(const Scalar& a, const Scalar& b) { return branch(a > b, b, a); }
Scalar max(const Scalar& a, const Scalar& b) { return branch(a > b, a, b); }
Scalar abs(const Scalar& a) { return branch(a > 0.0, a, -a); }
Scalar sign(const Scalar& a) { return branch(a > 0.0, 1.0, -1.0); }

// ------------------------------------------------------------------ Vector
Vector Vector::zero(int32_t n, const Scalar& seed) { return Vector(std::vector<Scalar>(n, seed.get_zero())); }
Vector Vector::segment(int32_t begin, int32_t n) const
{
    return Vector(std::vector<Scalar>(vals.begin() + begin, vals.begin() + begin + n));
}
void Vector::set_segment(int32_t begin, int32_t n, const Vector& o)
{
    for (int32_t i = 0; i < n; ++i) vals[begin + i] = o[i];
}
Scalar Vector::dot(const Vector& o) const
{
    Scalar s = vals[0] * o[0];
    for (int32_t i = 1; i < size(); ++i) s = s + vals[i] * o[i];
    return s;
}
Scalar Vector::cross2(const Vector& o) const { return vals[0] * o[1] - vals[1] * o[0]; }
Vector Vector::cross3(const Vector& o) const
{
    return Vector({vals[1] * o[2] - vals[2] * o[1], vals[2] * o[0] - vals[0] * o[2], vals[0] * o[1] - vals[1] * o[0]});
}
Scalar Vector::squared_norm() const { return dot(*this); }
Scalar Vector::norm() const { return squared_norm().sqrt(); }
Scalar Vector::stable_norm(const Scalar& eps) const { return (squared_norm() + eps).sqrt() - eps.sqrt(); }
Scalar Vector::stable_norm(double eps) const { return stable_norm(vals[0].make_constant(eps)); }
Vector Vector::normalized() const { return *this / norm(); }
Vector Vector::operator+(const Vector& o) const
{
    std::vector<Scalar> r(size());
    for (int32_t i = 0; i < size(); ++i) r[i] = vals[i] + o[i];
    return Vector(r);
}
Vector Vector::operator-(const Vector& o) const
{
    std::vector<Scalar> r(size());
    for (int32_t i = 0; i < size(); ++i) r[i] = vals[i] - o[i];
    return Vector(r);
}
Vector Vector::operator*(double v) const { return *this * vals[0].make_constant(v); }
Vector Vector::operator*(const Scalar& s) const
{
    std::vector<Scalar> r(size());
    for (int32_t i = 0; i < size(); ++i) r[i] = vals[i] * s;
    return Vector(r);
}
Vector Vector::operator/(double v) const { return *this / vals[0].make_constant(v); }
Vector Vector::operator/(const Scalar& s) const
{
    std::vector<Scalar> r(size());
    for (int32_t i = 0; i < size(); ++i) r[i] = vals[i] / s;
    return Vector(r);
}
Vector operator*(double v, const Vector& x) { return x * v; }
Vector operator*(const Scalar& s, const Vector& x)
{
    std::vector<Scalar> r(x.size());
    for (int32_t i = 0; i < x.size(); ++i) r[i] = s * x[i];
    return Vector(r);
}
Vector operator-(const Vector& x)
{
    std::vector<Scalar> r(x.size());
    for (int32_t i = 0; i < x.size(); ++i) r[i] = -x[i];
    return Vector(r);
}
Scalar dot(const Vector& a, const Vector& b) { return a.dot(b); }

// ------------------------------------------------------------------ Matrix
Matrix::Matrix(const std::vector<Scalar>& values, const std::array<int32_t, 2>& shape)
    : nrows(shape[0]), ncols(shape[1]), vals(values)
{
    if ((int32_t)values.size() != nrows * ncols) throw std::runtime_error("symx: Matrix size mismatch");
}
Matrix Matrix::zero(const std::array<int32_t, 2>& shape, const Scalar& seed)
{
    return Matrix(std::vector<Scalar>(shape[0] * shape[1], seed.get_zero()), shape);
}
Matrix Matrix::identity(int32_t n, const Scalar& seed)
{
    Matrix m = zero({n, n}, seed);
    for (int32_t i = 0; i < n; ++i) m(i, i) = seed.get_one();
    return m;
}
Matrix Matrix::block(int32_t r0, int32_t c0, int32_t nr, int32_t nc) const
{
    std::vector<Scalar> v;
    for (int32_t i = 0; i < nr; ++i)
        for (int32_t j = 0; j < nc; ++j) v.push_back((*this)(r0 + i, c0 + j));
    return Matrix(v, {nr, nc});
}
void Matrix::set_block(int32_t r0, int32_t c0, int32_t nr, int32_t nc, const Matrix& m)
{
    for (int32_t i = 0; i < nr; ++i)
        for (int32_t j = 0; j < nc; ++j) (*this)(r0 + i, c0 + j) = m(i, j);
}
Vector Matrix::row(int32_t i) const
{
    std::vector<Scalar> v(ncols);
    for (int32_t j = 0; j < ncols; ++j) v[j] = (*this)(i, j);
    return Vector(v);
}
Vector Matrix::col(int32_t j) const
{
    std::vector<Scalar> v(nrows);
    for (int32_t i = 0; i < nrows; ++i) v[i] = (*this)(i, j);
    return Vector(v);
}
void Matrix::set_row(int32_t i, const Vector& v)
{
    for (int32_t j = 0; j < ncols; ++j) (*this)(i, j) = v[j];
}
void Matrix::set_col(int32_t j, const Vector& v)
{
    for (int32_t i = 0; i < nrows; ++i) (*this)(i, j) = v[i];
}
Matrix Matrix::transpose() const
{
    std::vector<Scalar> v(vals.size());
    for (int32_t i = 0; i < nrows; ++i)
        for (int32_t j = 0; j < ncols; ++j) v[j * nrows + i] = (*this)(i, j);
    return Matrix(v, {ncols, nrows});
}
Scalar Matrix::det() const
{
    const Matrix& m = *this;
    if (nrows != ncols) throw std::runtime_error("symx: det of a non-square matrix");
    if (nrows == 1) return m(0, 0);
    if (nrows == 2) return m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0);
    if (nrows == 3) {
        return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0))
             + m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
    }
    if (nrows == 4) {
        Scalar s = m(0, 0).get_zero();
        for (int32_t j = 0; j < 4; ++j) {
            std::vector<Scalar> minor;
            for (int32_t r = 1; r < 4; ++r)
                for (int32_t c = 0; c < 4; ++c)
                    if (c != j) minor.push_back(m(r, c));
            const Scalar d = Matrix(minor, {3, 3}).det();
            s = (j % 2 == 0) ? s + m(0, j) * d : s - m(0, j) * d;
        }
        return s;
    }
    throw std::runtime_error("symx: det supports sizes up to 4");
}
Matrix Matrix::inv() const
{
    const Matrix& m = *this;
    if (nrows == 2) {
        const Scalar d = det();
        return Matrix({m(1, 1) / d, -m(0, 1) / d, -m(1, 0) / d, m(0, 0) / d}, {2, 2});
    }
    if (nrows == 3) {
        const Scalar d = det();
        std::vector<Scalar> v = {
            (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) / d, (m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2)) / d,
            (m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1)) / d, (m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2)) / d,
            (m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0)) / d, (m(0, 2) * m(1, 0) - m(0, 0) * m(1, 2)) / d,
            (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0)) / d, (m(0, 1) * m(2, 0) - m(0, 0) * m(2, 1)) / d,
            (m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0)) / d};
        return Matrix(v, {3, 3});
    }
    throw std::runtime_error("symx: inv supports 2x2 and 3x3");
}
Matrix Matrix::inv_sym() const
{
    Matrix r = inv();
    for (int32_t i = 0; i < nrows; ++i)
        for (int32_t j = 0; j < i; ++j) r(i, j) = r(j, i);
    return r;
}
Scalar Matrix::trace() const
{
    Scalar s = (*this)(0, 0);
    for (int32_t i = 1; i < nrows; ++i) s = s + (*this)(i, i);
    return s;
}
Scalar Matrix::frobenius_norm_sq() const
{
    Scalar s = vals[0] * vals[0];
    for (size_t i = 1; i < vals.size(); ++i) s = s + vals[i] * vals[i];
    return s;
}
Matrix Matrix::operator+(const Matrix& o) const
{
    std::vector<Scalar> v(vals.size());
    for (size_t i = 0; i < vals.size(); ++i) v[i] = vals[i] + o.vals[i];
    return Matrix(v, shape());
}
Matrix Matrix::operator-(const Matrix& o) const
{
    std::vector<Scalar> v(vals.size());
    for (size_t i = 0; i < vals.size(); ++i) v[i] = vals[i] - o.vals[i];
    return Matrix(v, shape());
}
Matrix Matrix::operator*(double s) const { return *this * vals[0].make_constant(s); }
Matrix Matrix::operator*(const Scalar& s) const
{
    std::vector<Scalar> v(vals.size());
    for (size_t i = 0; i < vals.size(); ++i) v[i] = vals[i] * s;
    return Matrix(v, shape());
}
Vector Matrix::operator*(const Vector& x) const
{
    std::vector<Scalar> v(nrows);
    for (int32_t i = 0; i < nrows; ++i) {
        Scalar s = (*this)(i, 0) * x[0];
        for (int32_t j = 1; j < ncols; ++j) s = s + (*this)(i, j) * x[j];
        v[i] = s;
    }
    return Vector(v);
}
Matrix Matrix::operator*(const Matrix& o) const
{
    if (ncols != o.nrows) throw std::runtime_error("symx: matrix product size mismatch");
    std::vector<Scalar> v(nrows * o.ncols);
    for (int32_t i = 0; i < nrows; ++i)
        for (int32_t j = 0; j < o.ncols; ++j) {
            Scalar s = (*this)(i, 0) * o(0, j);
            for (int32_t k = 1; k < ncols; ++k) s = s + (*this)(i, k) * o(k, j);
            v[i * o.ncols + j] = s;
        }
    return Matrix(v, {nrows, o.ncols});
}
Matrix Matrix::operator/(double s) const { return *this / vals[0].make_constant(s); }
Matrix Matrix::operator/(const Scalar& s) const
{
    std::vector<Scalar> v(vals.size());
    for (size_t i = 0; i < vals.size(); ++i) v[i] = vals[i] / s;
    return Matrix(v, shape());
}
Matrix operator*(double v, const Matrix& m) { return m * v; }
Matrix operator*(const Scalar& s, const Matrix& m) { return m * s; }
Matrix operator-(const Matrix& m) { return m * -1.0; }
Vector operator*(const Vector& v, const Matrix& m) { return m.transpose() * v; }
Matrix outer(const Vector& a, const Vector& b)
{
    std::vector<Scalar> v;
    for (int32_t i = 0; i < a.size(); ++i)
        for (int32_t j = 0; j < b.size(); ++j) v.push_back(a[i] * b[j]);
    return Matrix(v, {a.size(), b.size()});
}

// ------------------------------------------------------------------ Workspace
Scalar Workspace::make_scalar() { return Scalar(graph->new_symbol(), graph.get()); }
Vector Workspace::make_vector(int32_t n)
{
    std::vector<Scalar> v;
    for (int32_t i = 0; i < n; ++i) v.push_back(make_scalar());
    return Vector(v);
}
Matrix Workspace::make_matrix(const std::array<int32_t, 2>& shape)
{
    std::vector<Scalar> v;
    for (int32_t i = 0; i < shape[0] * shape[1]; ++i) v.push_back(make_scalar());
    return Matrix(v, shape);
}
std::vector<Scalar> Workspace::make_scalars(int32_t n)
{
    std::vector<Scalar> v;
    for (int32_t i = 0; i < n; ++i) v.push_back(make_scalar());
    return v;
}
std::vector<Vector> Workspace::make_vectors(int32_t size, int32_t n)
{
    std::vector<Vector> v;
    for (int32_t i = 0; i < n; ++i) v.push_back(make_vector(size));
    return v;
}
std::vector<Matrix> Workspace::make_matrices(const std::array<int32_t, 2>& shape, int32_t n)
{
    std::vector<Matrix> v;
    for (int32_t i = 0; i < n; ++i) v.push_back(make_matrix(shape));
    return v;
}

// ------------------------------------------------------------------ differentiation
namespace {
int32_t d_node(Expressions& g, int32_t f, int32_t wrt, DiffCache& cache)
{
    const int64_t key = ((int64_t)f << 32) | (uint32_t)wrt;
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const Node n = g[f];
    int32_t r = 0;
    auto D = [&](int32_t x) { return d_node(g, x, wrt, cache); };
    auto add = [&](int32_t a, int32_t b) { return g.add(Op::Add, a, b); };
    auto sub = [&](int32_t a, int32_t b) { return g.add(Op::Sub, a, b); };
    auto mul = [&](int32_t a, int32_t b) { return g.add(Op::Mul, a, b); };
    auto div = [&](int32_t a, int32_t b) { return g.add(Op::Div, a, b); };
    auto cst = [&](double v) { return g.constant(v); };
    switch (n.op) {
        case Op::Zero:
        case Op::One:
        case Op::Const: r = 0; break;
        case Op::Symbol: r = (f == wrt) ? 1 : 0; break;
        case Op::Add: r = add(D(n.a), D(n.b)); break;
        case Op::Sub: r = sub(D(n.a), D(n.b)); break;
        case Op::Neg: r = g.add(Op::Neg, D(n.a)); break;
        case Op::Mul: r = add(mul(D(n.a), n.b), mul(n.a, D(n.b))); break;
        case Op::Div: {
            // d(a/b) = (da - (a/b) db) / b; for the shared reciprocal f = 1/b: -f f db
            const int32_t da = D(n.a), db = D(n.b);
            if (n.a == 1) r = g.add(Op::Neg, mul(mul(f, f), db));
            else r = div(sub(da, mul(f, db)), n.b);
            break;
        }
        case Op::PowN: {
            const int32_t p = n.b;
            const int32_t base = (p - 1 == 1) ? n.a : g.add(Op::PowN, n.a, p - 1);
            r = mul(mul(cst((double)p), base), D(n.a));
            break;
        }
        case Op::PowF: r = mul(mul(cst(n.v), g.add(Op::PowF, n.a, -1, -1, n.v - 1.0)), D(n.a)); break;
        case Op::Sqrt: r = div(mul(cst(0.5), D(n.a)), f); break;
        case Op::Ln: r = div(D(n.a), n.a); break;
        case Op::Log10: r = div(D(n.a), mul(n.a, cst(std::log(10.0)))); break;
        case Op::Exp: r = mul(f, D(n.a)); break;
        case Op::Sin: r = mul(g.add(Op::Cos, n.a), D(n.a)); break;
        case Op::Cos: r = g.add(Op::Neg, mul(g.add(Op::Sin, n.a), D(n.a))); break;
        case Op::Tan: r = mul(add(1, mul(f, f)), D(n.a)); break;
        case Op::Asin: r = div(D(n.a), g.add(Op::Sqrt, sub(1, mul(n.a, n.a)))); break;
        case Op::Acos: r = g.add(Op::Neg, div(D(n.a), g.add(Op::Sqrt, sub(1, mul(n.a, n.a))))); break;
        case Op::Atan: r = div(D(n.a), add(1, mul(n.a, n.a))); break;
        case Op::Branch: r = g.add(Op::Branch, D(n.a), D(n.b), n.c); break;
    }
    cache.emplace(key, r);
    return r;
}
}  // namespace

Scalar diff(const Scalar& expr, const Scalar& wrt, DiffCache& cache)
{
    if (!wrt.is_symbol()) throw std::runtime_error("symx: diff with respect to a non-symbol");
    same_graph(expr, wrt);
    return Scalar(d_node(*expr.graph, expr.expr_id, wrt.expr_id, cache), expr.graph);
}
Scalar diff(const Scalar& expr, const Scalar& wrt)
{
    DiffCache c;
    return diff(expr, wrt, c);
}
Vector gradient(const Scalar& expr, const std::vector<Scalar>& wrt, DiffCache& cache)
{
    std::vector<Scalar> g;
    for (const Scalar& w : wrt) g.push_back(diff(expr, w, cache));
    return Vector(g);
}
Vector gradient(const Scalar& expr, const std::vector<Scalar>& wrt)
{
    DiffCache c;
    return gradient(expr, wrt, c);
}
Vector gradient(const Scalar& expr, const Vector& wrt) { return gradient(expr, wrt.values()); }
Matrix gradient(const Vector& f, const std::vector<Scalar>& wrt, bool symmetric, DiffCache& cache)
{
    const int32_t n = f.size(), m = (int32_t)wrt.size();
    std::vector<Scalar> v(n * m);
    for (int32_t i = 0; i < n; ++i)
        for (int32_t j = symmetric ? i : 0; j < m; ++j) v[i * m + j] = diff(f[i], wrt[j], cache);
    if (symmetric)
        for (int32_t i = 0; i < n; ++i)
            for (int32_t j = 0; j < i; ++j) v[i * m + j] = v[j * m + i];
    return Matrix(v, {n, m});
}
Matrix gradient(const Vector& f, const std::vector<Scalar>& wrt, bool symmetric)
{
    DiffCache c;
    return gradient(f, wrt, symmetric, c);
}
Matrix hessian(const Scalar& expr, const std::vector<Scalar>& wrt, DiffCache& cache)
{
    return gradient(gradient(expr, wrt, cache), wrt, true, cache);
}
Matrix hessian(const Scalar& expr, const std::vector<Scalar>& wrt)
{
    DiffCache c;
    return hessian(expr, wrt, c);
}
std::vector<Scalar> value_gradient(const Scalar& expr, const std::vector<Scalar>& wrt)
{
    std::vector<Scalar> out{expr};
    Vector g = gradient(expr, wrt);
    out.insert(out.end(), g.values().begin(), g.values().end());
    return out;
}
std::vector<Scalar> value_gradient_hessian(const Scalar& expr, const std::vector<Scalar>& wrt, DiffCache& cache)
{
    std::vector<Scalar> out{expr};
    Vector g = gradient(expr, wrt, cache);
    out.insert(out.end(), g.values().begin(), g.values().end());
    Matrix H = gradient(g, wrt, true, cache);
    out.insert(out.end(), H.values().begin(), H.values().end());
    return out;
}
std::vector<Scalar> value_gradient_hessian(const Scalar& expr, const std::vector<Scalar>& wrt)
{
    DiffCache c;
    return value_gradient_hessian(expr, wrt, c);
}
std::vector<Scalar> collect_scalars(const std::vector<Vector>& vectors)
{
    std::vector<Scalar> out;
    for (const Vector& v : vectors) out.insert(out.end(), v.values().begin(), v.values().end());
    return out;
}
std::vector<Scalar> collect_scalars(const std::vector<std::vector<Scalar>>& lists)
{
    std::vector<Scalar> out;
    for (const auto& l : lists) out.insert(out.end(), l.begin(), l.end());
    return out;
}

}  // namespace symx
