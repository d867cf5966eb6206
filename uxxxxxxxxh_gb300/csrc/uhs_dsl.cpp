// Stencil DSL reader: text -> program -> linear stencil descriptor.
// Grammar and precedence follow UHStencil/include/Parser/Parser.h (see
// include/uhs_dsl.h for the list); the reduction to a term list follows how
// MLIRGen lowers the expression tree to mulf/addf in evaluation order
// (lib/Parser/MLIRGen.cpp:357-480).
#include "../../include/uhs_dsl.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace uhs {
int set_error(int code, const char *fmt, ...);
}

namespace {

enum Tok {
    T_EOF = -1,
    T_IDENT = -2,
    T_NUMBER = -3,
    T_STENCIL = -4,
    T_FLOAT = -5,
    T_DOUBLE = -6,
    T_ITERATION = -7,
    T_MPITILE = -8,
    T_MPIHALO = -9,
    T_OPERATION = -10,
    T_DOMAIN = -11,
    T_KERNEL = -12,
    T_TILE = -13,
    T_SWCACHEAT = -14,
    T_EXPR = -15,
};

struct ParseError {
    std::string msg;
};

class Lexer {
public:
    Lexer(const char *text, std::string file) : s_(text), file_(std::move(file)) {}

    int cur() const { return tok_; }
    const std::string &ident() const { return ident_; }
    double number() const { return num_; }
    bool number_is_int() const { return num_int_; }
    int line() const { return tline_; }
    int col() const { return tcol_; }
    const std::string &file() const { return file_; }

    int next() {
        skip_space_and_comments();
        tline_ = line_;
        tcol_ = col_;
        const char c = peek();
        if (c == 0) return tok_ = T_EOF;
        if (std::isalpha((unsigned char)c)) {
            ident_.clear();
            while (std::isalnum((unsigned char)peek()) || peek() == '_') ident_ += get();
            static const std::map<std::string, int> kw = {
                {"stencil", T_STENCIL}, {"float", T_FLOAT},         {"double", T_DOUBLE},
                {"iteration", T_ITERATION}, {"mpiTile", T_MPITILE}, {"mpiHalo", T_MPIHALO},
                {"operation", T_OPERATION}, {"domain", T_DOMAIN},   {"kernel", T_KERNEL},
                {"tile", T_TILE},           {"swCacheAt", T_SWCACHEAT}, {"expr", T_EXPR}};
            auto it = kw.find(ident_);
            return tok_ = (it == kw.end() ? T_IDENT : it->second);
        }
        if (std::isdigit((unsigned char)c)) {
            std::string n;
            num_int_ = true;
            while (std::isdigit((unsigned char)peek()) || peek() == '.') {
                if (peek() == '.') num_int_ = false;
                n += get();
            }
            num_ = std::strtod(n.c_str(), nullptr);
            return tok_ = T_NUMBER;
        }
        return tok_ = (unsigned char)get();
    }

private:
    char peek() const { return s_[pos_]; }
    char get() {
        const char c = s_[pos_];
        if (c == 0) return c;
        ++pos_;
        if (c == '\n') {
            ++line_;
            col_ = 1;
        } else {
            ++col_;
        }
        return c;
    }
    void skip_space_and_comments() {
        for (;;) {
            while (peek() && std::isspace((unsigned char)peek())) get();
            if (peek() == '#') {
                while (peek() && peek() != '\n' && peek() != '\r') get();
                continue;
            }
            return;
        }
    }
    const char *s_;
    size_t pos_ = 0;
    int line_ = 1, col_ = 1, tline_ = 1, tcol_ = 1;
    int tok_ = T_EOF;
    std::string ident_;
    double num_ = 0;
    bool num_int_ = true;
    std::string file_;
};

// Expression tree.
struct Expr {
    enum Kind { Num, Access, Param, KernelRef, Bin } kind;
    double value = 0;           // Num
    std::string name;           // Access / Param / KernelRef
    std::vector<int64_t> idx;   // offsets (Access, KernelRef) or indices (Param)
    char op = 0;                // Bin
    std::unique_ptr<Expr> l, r; // Bin
};

struct Kernel {
    std::string name;
    std::vector<int64_t> tile;
    int swcache = -1;
    std::vector<std::pair<int64_t, int64_t>> domain;
    std::unique_ptr<Expr> expr;
};

struct Arg {
    std::string name;
    std::vector<int64_t> shape;
};

class Parser {
public:
    explicit Parser(Lexer &lx) : lx_(lx) {}

    void parse_module() {
        lx_.next();
        if (lx_.cur() != T_STENCIL) fail("stencil", "when parsing top level module");
        parse_stencil();
        if (lx_.cur() != T_EOF) fail("nothing", "at end of module");
    }

    std::string name;
    int dtype = UHS_F64;
    std::vector<Arg> args;
    int iteration = 0;
    std::vector<int64_t> mpi_tile;
    std::vector<std::pair<int64_t, int64_t>> mpi_halo;
    std::string operation;
    std::vector<Kernel> kernels;
    std::map<std::string, bool> is_struct;  // array name -> accessed with relative offsets

private:
    [[noreturn]] void fail(const char *expected, const char *ctx) {
        char buf[512];
        std::string got;
        if (lx_.cur() == T_IDENT) got = " '" + lx_.ident() + "'";
        else if (lx_.cur() == T_EOF) got = " end of input";
        else if (lx_.cur() > 0 && std::isprint(lx_.cur())) got = std::string(" '") + (char)lx_.cur() + "'";
        snprintf(buf, sizeof buf, "%s@%d:%d: expected '%s' %s but found%s", lx_.file().c_str(), lx_.line(),
                 lx_.col(), expected, ctx, got.c_str());
        throw ParseError{buf};
    }
    void expect(int t, const char *what, const char *ctx) {
        if (lx_.cur() != t) fail(what, ctx);
        lx_.next();
    }
    int64_t expect_int(const char *ctx) {
        if (lx_.cur() != T_NUMBER || !lx_.number_is_int()) fail("Integer", ctx);
        const int64_t v = (int64_t)lx_.number();
        lx_.next();
        return v;
    }
    std::vector<std::pair<int64_t, int64_t>> parse_ranges(const char *ctx) {
        std::vector<std::pair<int64_t, int64_t>> out;
        do {
            expect('[', "[", ctx);
            const int64_t a = expect_int(ctx);
            expect(',', ",", ctx);
            const int64_t b = expect_int(ctx);
            expect(']', "]", ctx);
            out.emplace_back(a, b);
        } while (lx_.cur() == '[');
        return out;
    }

    void parse_stencil() {
        lx_.next();
        if (lx_.cur() != T_IDENT) fail("stencil name", "in stencil define");
        name = lx_.ident();
        lx_.next();
        expect('(', "(", "in stencil define");
        if (lx_.cur() != ')') {
            if (lx_.cur() == T_FLOAT) dtype = UHS_F32;
            else if (lx_.cur() == T_DOUBLE) dtype = UHS_F64;
            else fail("float or double", "in stencil define");
            lx_.next();
            for (;;) {
                if (lx_.cur() != T_IDENT) fail("variable name", "in stencil define");
                Arg a;
                a.name = lx_.ident();
                lx_.next();
                do {
                    expect('[', "[", "in stencil define");
                    a.shape.push_back(expect_int("in stencil define"));
                    expect(']', "]", "in stencil define");
                } while (lx_.cur() == '[');
                if (a.shape.size() > 3) fail("at most 3 dimensions", "in stencil define");
                args.push_back(std::move(a));
                if (lx_.cur() != ',') break;
                lx_.next();
            }
            expect(')', ")", "in stencil define");
        }
        expect('{', "{", "in stencil define body");
        while (lx_.cur() != '}') {
            switch (lx_.cur()) {
                case T_ITERATION:
                    lx_.next();
                    expect('(', "(", "in stencil define body");
                    iteration = (int)expect_int("in stencil define body");
                    expect(')', ")", "in stencil define body");
                    break;
                case T_MPITILE:
                    lx_.next();
                    expect('(', "(", "in stencil define body");
                    for (;;) {
                        mpi_tile.push_back(expect_int("in stencil define body"));
                        if (lx_.cur() != ',') break;
                        lx_.next();
                    }
                    expect(')', ")", "in stencil define body");
                    break;
                case T_MPIHALO:
                    lx_.next();
                    expect('(', "(", "in stencil define body");
                    mpi_halo = parse_ranges("in stencil define body");
                    expect(')', ")", "in stencil define body");
                    break;
                case T_OPERATION:
                    lx_.next();
                    expect('(', "(", "in stencil define body");
                    if (lx_.cur() != T_IDENT) fail("kernel name", "in stencil define body");
                    operation = lx_.ident();
                    lx_.next();
                    expect(')', ")", "in stencil define body");
                    break;
                case T_KERNEL:
                    kernels.push_back(parse_kernel());
                    break;
                default:
                    fail("iteration, mpiTile, operation or kernel", "in stencil define body");
            }
        }
        lx_.next();
    }

    Kernel parse_kernel() {
        lx_.next();
        Kernel k;
        if (lx_.cur() != T_IDENT) fail("kernel name", "in kernel define");
        k.name = lx_.ident();
        lx_.next();
        expect('{', "{", "in kernel define body");
        while (lx_.cur() != '}') {
            switch (lx_.cur()) {
                case T_TILE:
                    lx_.next();
                    expect('(', "(", "in kernel define body");
                    for (;;) {
                        k.tile.push_back(expect_int("in kernel define body"));
                        if (lx_.cur() != ',') break;
                        lx_.next();
                    }
                    expect(')', ")", "in kernel define body");
                    break;
                case T_SWCACHEAT:
                    lx_.next();
                    expect('(', "(", "in kernel define body");
                    k.swcache = (int)expect_int("in kernel define body");
                    expect(')', ")", "in kernel define body");
                    break;
                case T_DOMAIN:
                    lx_.next();
                    expect('(', "(", "in kernel define body");
                    k.domain = parse_ranges("in kernel define body");
                    expect(')', ")", "in kernel define body");
                    break;
                case T_EXPR:
                    lx_.next();
                    expect('{', "{", "in kernel define body");
                    k.expr = parse_expression();
                    expect('}', "}", "in kernel define body");
                    break;
                default:
                    fail("tile, swCacheAt, domain, expr", "in kernel define body");
            }
        }
        lx_.next();
        return k;
    }

    static int prec(int t) {
        switch (t) {
            case '+':
            case '-':
                return 20;
            case '*':
            case '/':
                return 40;
            default:
                return -1;
        }
    }

    std::unique_ptr<Expr> parse_expression() { return parse_binop_rhs(0, parse_primary()); }

    std::unique_ptr<Expr> parse_binop_rhs(int min_prec, std::unique_ptr<Expr> lhs) {
        for (;;) {
            const int p = prec(lx_.cur());
            if (p < min_prec) return lhs;
            const char op = (char)lx_.cur();
            lx_.next();
            auto rhs = parse_primary();
            if (p < prec(lx_.cur())) rhs = parse_binop_rhs(p + 1, std::move(rhs));
            auto e = std::make_unique<Expr>();
            e->kind = Expr::Bin;
            e->op = op;
            e->l = std::move(lhs);
            e->r = std::move(rhs);
            lhs = std::move(e);
        }
    }

    std::unique_ptr<Expr> parse_primary() {
        switch (lx_.cur()) {
            case '-':
            case T_NUMBER: {
                double sign = 1;
                if (lx_.cur() == '-') {
                    sign = -1;
                    lx_.next();
                }
                if (lx_.cur() != T_NUMBER) fail("float point number", "in expr define");
                auto e = std::make_unique<Expr>();
                e->kind = Expr::Num;
                e->value = sign * lx_.number();
                lx_.next();
                return e;
            }
            case T_IDENT:
                return parse_identifier();
            case '(': {
                lx_.next();
                auto e = parse_expression();
                expect(')', ")", "to close expression with parentheses");
                return e;
            }
            default:
                fail("expression", "in expr define");
        }
    }

    std::unique_ptr<Expr> parse_identifier() {
        auto e = std::make_unique<Expr>();
        e->name = lx_.ident();
        lx_.next();
        if (lx_.cur() != '[') fail("[", "in expr define");
        int pattern = -1;  // 1 relative, 0 absolute
        while (lx_.cur() == '[') {
            lx_.next();
            int64_t v = 0;
            if (lx_.cur() == T_IDENT) {
                lx_.next();
                if (pattern == 0) fail("same index pattern", "in expr define");
                pattern = 1;
                if (lx_.cur() == '+' || lx_.cur() == '-') {
                    const int64_t s = lx_.cur() == '+' ? 1 : -1;
                    lx_.next();
                    v = s * expect_int("in expr define");
                } else if (lx_.cur() != ']') {
                    fail("+, -, ]", "in expr define");
                }
            } else if (lx_.cur() == T_NUMBER) {
                if (pattern == 1) fail("same index pattern", "in expr define");
                pattern = 0;
                v = expect_int("in expr define");
            } else {
                fail("x, y, z or Integer", "in expr define");
            }
            expect(']', "]", "in expr define");
            e->idx.push_back(v);
        }
        e->kind = pattern == 1 ? Expr::Access : Expr::Param;
        is_struct[e->name] = (pattern == 1);
        return e;
    }

    Lexer &lx_;
};

// Linear form of an expression: terms in evaluation order.
struct LTerm {
    int64_t o[3];
    double coef;
    int32_t param;  // >= 0: coefficient is params[param] * coef
};

struct Linear {
    std::vector<LTerm> terms;
    bool exact = true;   // left-to-right sum of the terms rounds like the tree
    bool single = false; // exactly one term produced by one rounding (or none)
};

}  // namespace

struct uhs_program {
    std::string name;
    int dtype = UHS_F64;
    int rank = 0;
    int64_t sizes[3] = {1, 1, 1};
    int64_t lb[3] = {0, 0, 0}, ub[3] = {1, 1, 1};
    int64_t tile[3] = {0, 0, 0};
    int ntile = 0;
    int iterations = 0;
    int nkernels = 0;
    int nparam_arrays = 0;
    bool exact = true;
    std::vector<uhs_term> terms;
    std::vector<double> params;
};

namespace {

struct Reducer {
    const Parser &P;
    std::string struct_name;
    int rank;
    std::map<std::string, const Kernel *> kernels;
    std::map<std::string, int> param_array;  // name -> index in arg list of param arrays
    int depth = 0;

    [[noreturn]] void unsupported(const std::string &m) { throw ParseError{"unsupported expression: " + m}; }

    static void pad(const std::vector<int64_t> &idx, int rank, int64_t o[3]) {
        o[0] = o[1] = o[2] = 0;
        for (int i = 0; i < (int)idx.size(); ++i) o[3 - rank + i] = idx[i];
    }

    // Constant value of a subtree that has no array access, or NAN flag.
    bool constant(const Expr &e, double *v) {
        if (e.kind == Expr::Num) {
            *v = e.value;
            return true;
        }
        if (e.kind == Expr::Bin) {
            double a, b;
            if (!constant(*e.l, &a) || !constant(*e.r, &b)) return false;
            switch (e.op) {
                case '+': *v = a + b; return true;
                case '-': *v = a - b; return true;
                case '*': *v = a * b; return true;
                case '/': *v = a / b; return true;
            }
        }
        return false;
    }

    Linear scale(Linear in, double c, int32_t param, bool product_rounds_once) {
        for (auto &t : in.terms) {
            if (param >= 0) {
                if (t.param >= 0) unsupported("product of two parameter values");
                t.param = param;
            }
            t.coef *= c;
        }
        in.exact = in.exact && in.single && product_rounds_once;
        return in;
    }

    Linear reduce(const Expr &e) {
        Linear L;
        switch (e.kind) {
            case Expr::Access: {
                if (e.name != struct_name) unsupported("access to a second grid '" + e.name + "'");
                if ((int)e.idx.size() != rank) unsupported("access '" + e.name + "' with wrong number of indices");
                LTerm t;
                pad(e.idx, rank, t.o);
                t.coef = 1.0;
                t.param = -1;
                L.terms.push_back(t);
                L.single = true;
                return L;
            }
            case Expr::KernelRef:
            case Expr::Param: {
                auto kit = kernels.find(e.name);
                if (kit != kernels.end()) {
                    // Producer kernel: inline its expression shifted by the offset.
                    if (++depth > 16) unsupported("kernel references nest too deep");
                    Linear in = reduce(*kit->second->expr);
                    --depth;
                    int64_t o[3];
                    pad(e.idx, rank, o);
                    for (auto &t : in.terms)
                        for (int i = 0; i < 3; ++i) t.o[i] += o[i];
                    in.exact = in.exact && in.single;
                    return in;
                }
                unsupported("parameter '" + e.name + "' outside a product with a grid access");
            }
            case Expr::Num:
                unsupported("constant term (the expression must be linear in the grid)");
            case Expr::Bin:
                break;
        }
        double c;
        if (e.op == '*' || e.op == '/') {
            // constant or parameter times linear part
            const Expr *lin = nullptr;
            double k = 1.0;
            int32_t param = -1;
            if (constant(*e.r, &c)) {
                lin = e.l.get();
                k = (e.op == '*') ? c : 1.0 / c;
            } else if (e.op == '*' && constant(*e.l, &c)) {
                lin = e.r.get();
                k = c;
            } else if (e.op == '*' && e.l->kind == Expr::Param && !kernels.count(e.l->name)) {
                lin = e.r.get();
                param = param_index(*e.l);
            } else if (e.op == '*' && e.r->kind == Expr::Param && !kernels.count(e.r->name)) {
                lin = e.l.get();
                param = param_index(*e.r);
            } else {
                unsupported("product of two grid-dependent values");
            }
            Linear in = reduce(*lin);
            const bool once = (e.op == '*') && (e.l->kind == Expr::Num || e.r->kind == Expr::Num ||
                                                 e.l->kind == Expr::Param || e.r->kind == Expr::Param);
            return scale(std::move(in), k, param, once);
        }
        if (constant(*e.l, &c) || constant(*e.r, &c)) unsupported("constant term (affine expression)");
        Linear a = reduce(*e.l), b = reduce(*e.r);
        if (e.op == '-')
            for (auto &t : b.terms) t.coef = -t.coef;
        Linear out;
        out.terms = std::move(a.terms);
        out.terms.insert(out.terms.end(), b.terms.begin(), b.terms.end());
        out.exact = a.exact && b.exact && b.single;
        out.single = false;
        return out;
    }

    int32_t param_index(const Expr &p) {
        auto it = param_array.find(p.name);
        if (it == param_array.end()) unsupported("unknown array '" + p.name + "'");
        if (p.idx.size() != 1) unsupported("parameter array '" + p.name + "' must have one index");
        // Parameter arrays are concatenated in argument order.
        return (int32_t)(it->second + p.idx[0]);
    }
};

int build_program(Parser &P, uhs_program *prog) {
    prog->name = P.name;
    prog->dtype = P.dtype;
    prog->iterations = P.iteration;
    prog->nkernels = (int)P.kernels.size();
    if (P.kernels.empty()) throw ParseError{"program '" + P.name + "' has no kernel"};
    const Kernel *op = nullptr;
    std::map<std::string, const Kernel *> kmap;
    for (const auto &k : P.kernels) {
        kmap[k.name] = &k;
        if (!k.expr) throw ParseError{"kernel '" + k.name + "' has no expr"};
    }
    if (P.operation.empty()) op = &P.kernels.back();
    else {
        auto it = kmap.find(P.operation);
        if (it == kmap.end()) throw ParseError{"operation kernel '" + P.operation + "' is not defined"};
        op = it->second;
    }
    // The struct array is the one accessed with relative offsets.
    std::string sname;
    const Arg *sarg = nullptr;
    std::map<std::string, int> param_base;
    int pbase = 0;
    for (const auto &a : P.args) {
        auto it = P.is_struct.find(a.name);
        const bool is_struct = it != P.is_struct.end() && it->second;
        if (is_struct) {
            if (sarg) throw ParseError{"programs with more than one grid are not supported"};
            sarg = &a;
            sname = a.name;
        } else {
            param_base[a.name] = pbase;
            int64_t n = 1;
            for (auto d : a.shape) n *= d;
            pbase += (int)n;
            prog->nparam_arrays++;
        }
    }
    if (!sarg) throw ParseError{"no grid argument is accessed with relative offsets"};
    prog->rank = (int)sarg->shape.size();
    if (prog->rank != 2 && prog->rank != 3) throw ParseError{"grids must have rank 2 or 3"};
    for (int i = 0; i < prog->rank; ++i) prog->sizes[3 - prog->rank + i] = sarg->shape[i];
    if ((int)op->domain.size() != prog->rank)
        throw ParseError{"domain of kernel '" + op->name + "' does not match the grid's rank"};
    for (int i = 0; i < prog->rank; ++i) {
        prog->lb[3 - prog->rank + i] = op->domain[i].first;
        prog->ub[3 - prog->rank + i] = op->domain[i].second;
    }
    prog->ntile = (int)std::min<size_t>(op->tile.size(), 3);
    for (int i = 0; i < prog->ntile; ++i) prog->tile[3 - prog->ntile + i] = op->tile[i];
    // A reference to another kernel uses relative indices, so the parser
    // tagged it as a grid access under the kernel's name; retag it.
    Reducer R{P, sname, prog->rank, {}, param_base, 0};
    for (const auto &k : P.kernels)
        if (&k != op) R.kernels[k.name] = &k;
    // Re-tag accesses to kernel names: reduce() resolves Access nodes whose
    // name is a kernel through the KernelRef path.
    struct Retag {
        const std::map<std::string, const Kernel *> &km;
        void operator()(Expr &e) const {
            if (e.kind == Expr::Access && km.count(e.name)) e.kind = Expr::KernelRef;
            if (e.l) (*this)(*e.l);
            if (e.r) (*this)(*e.r);
        }
    };
    for (auto &k : P.kernels) Retag{R.kernels}(*k.expr);
    Linear L = R.reduce(*op->expr);
    if (L.terms.empty()) throw ParseError{"operation kernel has no grid terms"};
    if ((int)L.terms.size() > UHS_MAX_TERMS) throw ParseError{"expression has more than UHS_MAX_TERMS terms"};
    prog->exact = L.exact;
    for (const auto &t : L.terms) {
        uhs_term u;
        u.dz = (int32_t)t.o[0];
        u.dy = (int32_t)t.o[1];
        u.dx = (int32_t)t.o[2];
        u.param = t.param;
        u.coef = t.coef;
        if (t.param >= 0 && t.coef != 1.0) prog->exact = false;
        prog->terms.push_back(u);
    }
    prog->params.assign(pbase, 0.0);
    return UHS_OK;
}

}  // namespace

extern "C" {

int uhs_dsl_parse(const char *text, const char *filename, uhs_program **out) {
    if (!text || !out) return uhs::set_error(UHS_EINVAL, "text and out must be non-NULL");
    *out = nullptr;
    Lexer lx(text, filename ? filename : "<dsl>");
    Parser P(lx);
    auto prog = std::make_unique<uhs_program>();
    try {
        P.parse_module();
        build_program(P, prog.get());
    } catch (const ParseError &e) {
        const bool unsup = e.msg.rfind("unsupported", 0) == 0 || e.msg.find("not supported") != std::string::npos;
        return uhs::set_error(unsup ? UHS_EUNSUPPORTED : UHS_EPARSE, "%s", e.msg.c_str());
    }
    *out = prog.release();
    return UHS_OK;
}

void uhs_program_free(uhs_program *p) { delete p; }

const char *uhs_program_name(const uhs_program *p) { return p ? p->name.c_str() : ""; }

int uhs_program_desc(const uhs_program *p, uhs_stencil_desc *d, int64_t sizes[3]) {
    if (!p || !d) return uhs::set_error(UHS_EINVAL, "program and desc must be non-NULL");
    std::memset(d, 0, sizeof *d);
    d->rank = p->rank;
    d->dtype = p->dtype;
    for (int i = 0; i < 3; ++i) {
        d->lb[i] = p->lb[i];
        d->ub[i] = p->ub[i];
        if (sizes) sizes[i] = p->sizes[i];
    }
    d->nterms = (int32_t)p->terms.size();
    d->terms = p->terms.data();
    d->iterations = p->iterations;
    d->params = p->params.empty() ? nullptr : p->params.data();
    d->nparams = (int32_t)p->params.size();
    return UHS_OK;
}

int uhs_program_exact_order(const uhs_program *p) { return p && p->exact ? 1 : 0; }

int uhs_program_tile(const uhs_program *p, int64_t tile[3]) {
    if (!p) return 0;
    for (int i = 0; i < 3; ++i) tile[i] = p->tile[i];
    return p->ntile;
}

int uhs_program_num_kernels(const uhs_program *p) { return p ? p->nkernels : 0; }
int uhs_program_num_param_arrays(const uhs_program *p) { return p ? p->nparam_arrays : 0; }

int uhs_program_set_params(uhs_program *p, const double *v, int32_t n) {
    if (!p || (!v && n > 0)) return uhs::set_error(UHS_EINVAL, "program and values must be non-NULL");
    if (n != (int32_t)p->params.size())
        return uhs::set_error(UHS_EINVAL, "program has %zu parameter values, %d given", p->params.size(), n);
    for (int32_t i = 0; i < n; ++i) p->params[i] = v[i];
    return UHS_OK;
}

}  // extern "C"
