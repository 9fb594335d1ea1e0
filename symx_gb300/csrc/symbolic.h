// Symbolic front end: expression DAG, Scalar/Vector/Matrix algebra and symbolic
// differentiation, with the user-facing names of the reference SymX
// (symx/src/symbol/{Workspace,Scalar,Vector,Matrix,diff}.h) so that energy
// definitions written against it compile unchanged.
//
// The DAG is a flat array of nodes with hash-consing: building the same
// (op, operands, constant) twice returns the same node, which is the common
// subexpression elimination the code generator relies on.  Symbols are numbered
// in creation order; that number is the symbol's input slot in generated code
// (the reference's contract, symx/src/compile/Compiled.cpp:86-90).
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace symx {

enum class Op : int32_t {
    Zero = 0, One, Const, Symbol,
    Add, Sub, Mul, Div, Neg,
    PowN, PowF, Sqrt, Ln, Log10, Exp, Sin, Cos, Tan, Asin, Acos, Atan,
    Branch,  // c > 0 ? a : b
};

struct Node {
    Op op;
    int32_t a = -1, b = -1, c = -1;  // operands (PowN: b is the integer exponent)
    double v = 0.0;                   // Const value, PowF exponent
};

// Flat expression graph.  Node 0 is zero, node 1 is one.
class Expressions {
public:
    Expressions();
    int32_t add(Op op, int32_t a = -1, int32_t b = -1, int32_t c = -1, double v = 0.0);
    int32_t constant(double v);
    int32_t new_symbol();
    const Node& operator[](int32_t i) const { return nodes_[i]; }
    int32_t size() const { return (int32_t)nodes_.size(); }
    int32_t n_symbols() const { return n_symbols_; }
    int32_t symbol_node(int32_t symbol_idx) const { return symbol_nodes_[symbol_idx]; }
    // Input slot of a symbol node (its creation index).
    int32_t symbol_index(int32_t node) const { return (int32_t)nodes_[node].v; }
    // Numeric evaluation with the symbol values set by Scalar::set_value.
    double eval(int32_t node) const;
    void set_symbol_value(int32_t symbol_idx, double v);
    // Stable 64-bit hash of the sub-graph needed by `roots` (FNV-1a over node records in
    // dependency order), used for the generated-kernel cache key.
    uint64_t hash(const std::vector<int32_t>& roots) const;

private:
    struct Key {
        int32_t op, a, b, c;
        uint64_t v;
        bool operator==(const Key& o) const { return op == o.op && a == o.a && b == o.b && c == o.c && v == o.v; }
    };
    struct KeyHash {
        size_t operator()(const Key& k) const;
    };
    std::vector<Node> nodes_;
    std::vector<int32_t> symbol_nodes_;
    std::vector<double> symbol_values_;
    std::unordered_map<Key, int32_t, KeyHash> map_;
    int32_t n_symbols_ = 0;
};

class Scalar {
public:
    Scalar() = default;
    Scalar(int32_t id, Expressions* g) : expr_id(id), graph(g) {}

    int32_t expr_id = -1;
    Expressions* graph = nullptr;

    Scalar operator+(const Scalar& o) const;
    Scalar operator-(const Scalar& o) const;
    Scalar operator*(const Scalar& o) const;
    Scalar operator/(const Scalar& o) const;
    Scalar operator+(double v) const;
    Scalar operator-(double v) const;
    Scalar operator*(double v) const;
    Scalar operator/(double v) const;
    void operator+=(const Scalar& o) { *this = *this + o; }
    void operator-=(const Scalar& o) { *this = *this - o; }
    void operator*=(const Scalar& o) { *this = *this * o; }
    void operator/=(const Scalar& o) { *this = *this / o; }
    void operator+=(double v) { *this = *this + v; }
    void operator-=(double v) { *this = *this - v; }
    void operator*=(double v) { *this = *this * v; }
    void operator/=(double v) { *this = *this / v; }

    Scalar powN(int32_t n) const;
    Scalar powF(double p) const;
    Scalar inv() const;
    Scalar sqrt() const;
    Scalar log() const { return ln(); }
    Scalar ln() const;
    Scalar log10() const;
    Scalar exp() const;
    Scalar sin() const;
    Scalar cos() const;
    Scalar tan() const;
    Scalar asin() const;
    Scalar acos() const;
    Scalar atan() const;

    bool is_zero() const { return expr_id == 0; }
    bool is_one() const { return expr_id == 1; }
    bool is_symbol() const { return graph && (*graph)[expr_id].op == Op::Symbol; }
    bool is_constant() const;
    int32_t get_symbol_idx() const { return graph->symbol_index(expr_id); }
    void set_value(double v) const;
    double eval() const { return graph->eval(expr_id); }
    // Reproducible hash of the part of the graph this expression depends on (hex string),
    // the cache id of a Compiled<T> (reference: symx/src/symbol/Scalar.h:75).
    std::string get_checksum() const;
    Scalar make_constant(double v) const { return Scalar(graph->constant(v), graph); }
    Scalar get_zero() const { return Scalar(0, graph); }
    Scalar get_one() const { return Scalar(1, graph); }
};

Scalar operator+(double v, const Scalar& s);
Scalar operator-(double v, const Scalar& s);
Scalar operator*(double v, const Scalar& s);
Scalar operator/(double v, const Scalar& s);
Scalar operator-(const Scalar& s);
Scalar powN(const Scalar& s, int32_t n);
Scalar powF(const Scalar& s, double p);
Scalar sqrt(const Scalar& s);
Scalar log(const Scalar& s);
Scalar ln(const Scalar& s);
Scalar log10(const Scalar& s);
Scalar exp(const Scalar& s);
Scalar sin(const Scalar& s);
Scalar cos(const Scalar& s);
Scalar tan(const Scalar& s);
Scalar asin(const Scalar& s);
Scalar acos(const Scalar& s);
Scalar atan(const Scalar& s);
// branch(cond, p, n) = cond > 0 ? p : n.  `a > b` is the condition a - b (as in the
// reference, symx/src/symbol/Scalar.cpp:532-559).
Scalar branch(const Scalar& cond, const Scalar& pos, const Scalar& neg);
Scalar branch(const Scalar& cond, double pos, const Scalar& neg);
Scalar branch(const Scalar& cond, const Scalar& pos, double neg);
Scalar branch(const Scalar& cond, double pos, double neg);
Scalar operator>(const Scalar& a, const Scalar& b);
Scalar operator<(const Scalar& a, const Scalar& b);
Scalar operator>(const Scalar& a, double b);
Scalar operator<(const Scalar& a, double b);
Scalar operator>(double a, const Scalar& b);
Scalar operator<(double a, const Scalar& b);
Scalar min(const Scalar& a, const Scalar& b);
Scalar max(const Scalar& a, const Scalar& b);
Scalar abs(const Scalar& a);
Scalar sign(const Scalar& a);

class Vector {
public:
    Vector() = default;
    Vector(const std::vector<Scalar>& values) : vals(values) {}
    static Vector zero(int32_t n, const Scalar& seed);

    int32_t size() const { return (int32_t)vals.size(); }
    std::vector<Scalar>& values() { return vals; }
    const std::vector<Scalar>& values() const { return vals; }
    Scalar& operator[](int32_t i) { return vals[i]; }
    const Scalar& operator[](int32_t i) const { return vals[i]; }
    Scalar& operator()(int32_t i) { return vals[i]; }
    const Scalar& operator()(int32_t i) const { return vals[i]; }
    Vector segment(int32_t begin, int32_t n) const;
    void set_segment(int32_t begin, int32_t n, const Vector& o);
    template <typename T>
    void set_values(const T& v) { for (int32_t i = 0; i < size(); ++i) vals[i].set_value(v[i]); }

    Scalar dot(const Vector& o) const;
    Scalar cross2(const Vector& o) const;
    Vector cross3(const Vector& o) const;
    Scalar squared_norm() const;
    Scalar norm() const;
    Scalar stable_norm(double eps) const;
    Scalar stable_norm(const Scalar& eps) const;
    Vector normalized() const;
    void normalize() { *this = normalized(); }

    Vector operator+(const Vector& o) const;
    Vector operator-(const Vector& o) const;
    Vector operator*(double v) const;
    Vector operator*(const Scalar& s) const;
    Vector operator/(double v) const;
    Vector operator/(const Scalar& s) const;
    void operator+=(const Vector& o) { *this = *this + o; }
    void operator-=(const Vector& o) { *this = *this - o; }
    void operator*=(double v) { *this = *this * v; }
    void operator*=(const Scalar& s) { *this = *this * s; }
    void operator/=(double v) { *this = *this / v; }
    void operator/=(const Scalar& s) { *this = *this / s; }

private:
    std::vector<Scalar> vals;
};
Vector operator*(double v, const Vector& x);
Vector operator*(const Scalar& s, const Vector& x);
Vector operator-(const Vector& x);
Scalar dot(const Vector& a, const Vector& b);

class Matrix {
public:
    Matrix() = default;
    Matrix(const std::vector<Scalar>& values, const std::array<int32_t, 2>& shape);
    static Matrix zero(const std::array<int32_t, 2>& shape, const Scalar& seed);
    static Matrix identity(int32_t n, const Scalar& seed);

    int32_t rows() const { return nrows; }
    int32_t cols() const { return ncols; }
    std::array<int32_t, 2> shape() const { return {nrows, ncols}; }
    std::vector<Scalar>& values() { return vals; }
    const std::vector<Scalar>& values() const { return vals; }
    Scalar& operator()(int32_t i, int32_t j) { return vals[i * ncols + j]; }
    const Scalar& operator()(int32_t i, int32_t j) const { return vals[i * ncols + j]; }
    template <typename T>
    void set_values_row_major(const T& v)
    {
        for (int32_t i = 0; i < nrows; ++i)
            for (int32_t j = 0; j < ncols; ++j) (*this)(i, j).set_value(v(i, j));
    }

    Matrix block(int32_t r0, int32_t c0, int32_t nr, int32_t nc) const;
    void set_block(int32_t r0, int32_t c0, int32_t nr, int32_t nc, const Matrix& m);
    Vector row(int32_t i) const;
    Vector col(int32_t j) const;
    void set_row(int32_t i, const Vector& v);
    void set_col(int32_t j, const Vector& v);
    Matrix transpose() const;
    Scalar det() const;
    Matrix inv() const;
    Matrix inv_sym() const;
    Scalar trace() const;
    Scalar frobenius_norm_sq() const;
    Matrix dot(const Matrix& o) const { return *this * o; }
    Vector dot(const Vector& v) const { return *this * v; }

    Matrix operator+(const Matrix& o) const;
    Matrix operator-(const Matrix& o) const;
    Matrix operator*(double v) const;
    Matrix operator*(const Scalar& s) const;
    Vector operator*(const Vector& v) const;
    Matrix operator*(const Matrix& o) const;
    Matrix operator/(double v) const;
    Matrix operator/(const Scalar& s) const;
    void operator+=(const Matrix& o) { *this = *this + o; }
    void operator-=(const Matrix& o) { *this = *this - o; }
    void operator*=(double v) { *this = *this * v; }
    void operator*=(const Scalar& s) { *this = *this * s; }
    void operator/=(double v) { *this = *this / v; }
    void operator/=(const Scalar& s) { *this = *this / s; }

private:
    int32_t nrows = 0, ncols = 0;
    std::vector<Scalar> vals;
};
Matrix operator*(double v, const Matrix& m);
Matrix operator*(const Scalar& s, const Matrix& m);
Matrix operator-(const Matrix& m);
Vector operator*(const Vector& v, const Matrix& m);
Matrix outer(const Vector& a, const Vector& b);

// Symbol factory over one expression graph (reference: symx/src/symbol/Workspace.h:19-47).
class Workspace {
public:
    Workspace() : graph(std::make_shared<Expressions>()) {}
    Scalar make_scalar();
    Vector make_vector(int32_t n);
    Matrix make_matrix(const std::array<int32_t, 2>& shape);
    std::vector<Scalar> make_scalars(int32_t n);
    std::vector<Vector> make_vectors(int32_t size, int32_t n);
    std::vector<Matrix> make_matrices(const std::array<int32_t, 2>& shape, int32_t n);
    Scalar get_zero() { return Scalar(0, graph.get()); }
    Scalar get_one() { return Scalar(1, graph.get()); }
    Scalar make_constant(double v) { return Scalar(graph->constant(v), graph.get()); }
    Vector get_zero_vector(int32_t n) { return Vector::zero(n, get_zero()); }
    Matrix get_zero_matrix(const std::array<int32_t, 2>& shape) { return Matrix::zero(shape, get_zero()); }
    Matrix get_identity_matrix(int32_t n) { return Matrix::identity(n, get_zero()); }
    int32_t get_n_symbols() const { return graph->n_symbols(); }
    Expressions& get_expression_graph() { return *graph; }
    const Expressions& get_expression_graph() const { return *graph; }
    std::shared_ptr<Expressions> graph;
};

// Differentiation (reference: symx/src/symbol/diff.h:21-47).  The cache memoises
// d(node)/d(symbol) across calls on the same graph.
using DiffCache = std::unordered_map<int64_t, int32_t>;
Scalar diff(const Scalar& expr, const Scalar& wrt);
Scalar diff(const Scalar& expr, const Scalar& wrt, DiffCache& cache);
Vector gradient(const Scalar& expr, const std::vector<Scalar>& wrt);
Vector gradient(const Scalar& expr, const std::vector<Scalar>& wrt, DiffCache& cache);
Vector gradient(const Scalar& expr, const Vector& wrt);
// Jacobian of a vector; with `symmetric` only the upper triangle is differentiated and
// mirrored (the Hessian case).
Matrix gradient(const Vector& f, const std::vector<Scalar>& wrt, bool symmetric);
Matrix gradient(const Vector& f, const std::vector<Scalar>& wrt, bool symmetric, DiffCache& cache);
Matrix hessian(const Scalar& expr, const std::vector<Scalar>& wrt);
Matrix hessian(const Scalar& expr, const std::vector<Scalar>& wrt, DiffCache& cache);
// [E, g_0..g_{n-1}, H row-major] (reference output layout, symx/src/symbol/diff.cpp:209-214).
std::vector<Scalar> value_gradient(const Scalar& expr, const std::vector<Scalar>& wrt);
std::vector<Scalar> value_gradient_hessian(const Scalar& expr, const std::vector<Scalar>& wrt);
std::vector<Scalar> value_gradient_hessian(const Scalar& expr, const std::vector<Scalar>& wrt, DiffCache& cache);

std::vector<Scalar> collect_scalars(const std::vector<Vector>& vectors);
std::vector<Scalar> collect_scalars(const std::vector<std::vector<Scalar>>& lists);

}  // namespace symx
