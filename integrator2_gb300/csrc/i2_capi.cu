// i2_capi.cu -- host side of the library behind the C-ABI declared in include/integrator2_gb300.h.
//
// Handles own their device buffers (RAII, no shallow copies).  Every CUDA call is checked and
// turned into an i2_status with a thread-local message; nothing calls exit().
#include "integrator2_gb300.h"
#include "i2_engine.h"
#include "i2_host.h"
#include "i2_pairs.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <memory>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

using i2::DevBuf;
using i2::Failure;

thread_local std::string g_error;

template <class F>
i2_status guarded(F &&f)
{
    try {
        f();
        g_error.clear();
        return I2_OK;
    } catch (const Failure &x) {
        g_error = x.msg;
        return x.code;
    } catch (const std::bad_alloc &) {
        g_error = "host allocation failed";
        return I2_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &x) {
        g_error = x.what();
        return I2_ERR_INVALID_ARGUMENT;
    }
}

// ------------------------------------------------------------------ quadrature
struct Rule {
    std::vector<double> c, w;
    int order;
};

// The reference's built-in rules (src/QuadratureFormula3d.cuh:34-213): Cowper's published
// tables, stored as (L1, L2, w) rows in the published point order.
const Rule *builtin_rule(int npoints)
{
    static const std::unordered_map<int, Rule> rules = [] {
        std::unordered_map<int, Rule> r;
        auto add = [&](int n, int order, std::initializer_list<double> rows) {
            Rule q;
            q.order = order;
            std::vector<double> v(rows);
            for (size_t k = 0; k + 2 < v.size(); k += 3) {
                q.c.push_back(v[k]);
                q.c.push_back(v[k + 1]);
                q.w.push_back(v[k + 2]);
            }
            r[n] = q;
        };
        const double t = 0.3333333333333333;
        add(1, 2, {t, t, 1.0});
        add(3, 2, {0.1666666666666667, 0.1666666666666667, 0.3333333333333333, 0.6666666666666667, 0.1666666666666667,
                   0.3333333333333333, 0.1666666666666667, 0.6666666666666667, 0.3333333333333333});
        add(4, 3, {t, t, -0.5625, 0.6, 0.2, 0.5208333333333333, 0.2, 0.6, 0.5208333333333333, 0.2, 0.2, 0.5208333333333333});
        {
            const double a = 0.816847572980459, b = 0.091576213509771, wa = 0.109951743655322;
            const double c = 0.445948490915965, d = 0.108103018168070, wc = 0.223381589678011;
            add(6, 4, {a, b, wa, b, a, wa, b, b, wa, c, d, wc, d, c, wc, c, c, wc});
        }
        {
            const double a = 0.101286507323456, b = 0.797426985353087, wa = 0.125939180544827;
            const double c = 0.470142064105115, d = 0.059715871789770, wc = 0.132394152788506;
            add(7, 5, {t, t, 0.225, a, b, wa, b, a, wa, a, a, wa, c, d, wc, d, c, wc, c, c, wc});
        }
        {
            const double a = 0.437525248383384, b = 0.124949503233232, wa = 0.205950504760887;
            const double c = 0.797112651860071, d = 0.165409927389841, e = 0.037477420750088, wc = 0.063691414286223;
            add(9, 5, {a, b, wa, b, a, wa, a, a, wa, c, d, wc, d, c, wc, c, e, wc, e, c, wc, d, e, wc, e, d, wc});
        }
        {
            const double a = 0.873821971016996, b = 0.063089014491502, wa = 0.050844906370207;
            const double c = 0.501426509658179, d = 0.249286745170910, wc = 0.116786275726379;
            const double e = 0.636502499121399, f = 0.310352451033785, g = 0.053145049844816, we = 0.082851075618374;
            add(12, 6, {a, b, wa, b, a, wa, b, b, wa, c, d, wc, d, c, wc, d, d, wc,
                        e, f, we, f, e, we, e, g, we, g, e, we, f, g, we, g, f, we});
        }
        {
            const double a = 0.479308067841923, b = 0.260345966079038, wa = 0.175615257433204;
            const double c = 0.869739794195598, d = 0.065130102902216, wc = 0.053347235608839;
            const double e = 0.638444188569809, f = 0.312865496004875, g = 0.048690315425316, we = 0.077113760890257;
            const double m = 0.333333333333333;
            add(13, 7, {m, m, -0.149570044467670, a, b, wa, b, a, wa, b, b, wa, c, d, wc, d, c, wc, d, d, wc,
                        e, f, we, f, e, we, e, g, we, g, e, we, f, g, we, g, f, we});
        }
        return r;
    }();
    auto it = rules.find(npoints);
    return it == rules.end() ? nullptr : &it->second;
}

// Gauss-Legendre nodes/weights on [0, 1] (Newton iteration on the Legendre recurrence)
void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w)
{
    x.resize(n);
    w.resize(n);
    for (int k = 0; k < n; ++k) {
        double z = std::cos(M_PI * (k + 0.75) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = 0.0;
            for (int m = 1; m <= n; ++m) {
                const double p2 = p1;
                p1 = p0;
                p0 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p2) / m;
            }
            dp = n * (z * p0 - p1) / (z * z - 1.0);
            const double dz = p0 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[n - 1 - k] = 0.5 * (z + 1.0);
        w[n - 1 - k] = 1.0 / ((1.0 - z * z) * dp * dp);
    }
}

// ------------------------------------------------------------------ .dat reader
// Reference semantics (src/Mesh3d.cu:159-217): header 'nv nc', nv lines 'idx x y z', then
// elements 'idx type ...'; type 203 = triangle 'a b c' (1-based); other types consume two more
// tokens and lower the cell count; the kept cells are the first (count - skipped) triangles.
// With trailing whitespace the reference's read loop turns once more on a failed read that
// keeps the last type value: a triangle type changes nothing, any other type skips one more.
bool read_dat(const std::string &path, double scale, std::vector<double> &V, std::vector<int> &C, std::string &err)
{
    std::ifstream f(path);
    if (!f.is_open()) {
        err = "cannot open " + path;
        return false;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    std::istringstream in(text);
    std::vector<std::string> tok;
    std::string s;
    while (in >> s) tok.push_back(s);
    if (tok.size() < 2) {
        err = "truncated mesh header";
        return false;
    }
    size_t p = 0;
    const long nv = std::stol(tok[p++]);
    long nc = std::stol(tok[p++]);
    if (nv < 0 || nc < 0 || p + 4 * (size_t)nv > tok.size()) {
        err = "bad vertex section";
        return false;
    }
    V.resize(3 * nv);
    for (long k = 0; k < nv; ++k) {
        ++p;
        for (int d = 0; d < 3; ++d) V[3 * k + d] = scale * std::stod(tok[p++]);
    }
    std::vector<int> cells;
    long last_type = 0;
    while (p < tok.size()) {
        last_type = p + 1 < tok.size() ? std::stol(tok[p + 1]) : 0;
        if (last_type == 203) {
            if (p + 4 >= tok.size()) {
                err = "truncated triangle";
                return false;
            }
            for (int d = 0; d < 3; ++d) cells.push_back(std::stoi(tok[p + 2 + d]) - 1);
            p += 5;
        } else {
            --nc;
            p += 4;
        }
    }
    if (!text.empty() && std::isspace((unsigned char)text.back()) && last_type != 203) --nc;
    if (nc < 0) nc = 0;
    if ((long)cells.size() / 3 < nc) nc = cells.size() / 3;
    cells.resize(3 * nc);
    for (int c : cells)
        if (c < 0 || c >= nv) {
            err = "cell references a missing vertex";
            return false;
        }
    C.swap(cells);
    return true;
}

} // namespace

// ------------------------------------------------------------------ handles
struct i2_mesh {
    std::vector<double> V;
    std::vector<int> C;
    std::vector<double> normals, measures, centres;
    std::vector<int> lists[4];  // unordered (i < j) pairs per class, flattened (i, j)
    bool host_lists = true;     // lists[] hold the current lists (a device build may skip the host copy)
    i2::DevicePairLists dlists; // the same lists on the device
    bool dlists_ok = false;     // dlists hold the current lists
    bool prepared = false;   // host geometry and pair lists ready
    bool on_device = false;  // vertices, cells and panels uploaded (first run)
    double near_factor = 3.0;
    DevBuf<double> dV;
    DevBuf<int> dC;
    DevBuf<i2::Panel> dPanels;
    DevBuf<i2::PanelF> dPanelsF;
    int nv() const { return (int)(V.size() / 3); }
    int nc() const { return (int)(C.size() / 3); }
};

struct i2_integrator {
    const i2_mesh *mesh = nullptr;
    std::vector<double> coords, weights;
    int order = 7;
    i2::RunConfig cfg;
    int precision = I2_PRECISION_FP64;
    int pot_nu = 10, pot_nv = 8, pot_grade = 3;
    // points per edge piece of the self-pair rule; 0 (default): the closed form in both precisions
    // (exact; the edge rule converges slowly on distorted cells: 8e-6 at 12 points on a sphere
    // jittered by 0.3 h)
    int pot_nself = 0;
    int self_points() const { return pot_nself > 0 ? pot_nself : 0; }
    i2::QuadTables tables() const { return tables(precision == I2_PRECISION_MIXED); }
    // mixed: the tables of the mixed-precision form (tier 2b's check rule 20 x 20, below)
    i2::QuadTables tables(bool mixed) const
    {
        i2::QuadTables Q;
        std::memset(&Q, 0, sizeof Q);
        Q.npts = (int)weights.size();
        for (int g = 0; g < Q.npts; ++g) {
            Q.L1[g] = coords[2 * g];
            Q.L2[g] = coords[2 * g + 1];
            Q.L3[g] = 1.0 - coords[2 * g] - coords[2 * g + 1];
            Q.w[g] = weights[g];
        }
        Q.order = order;
        Q.pow2p = (double)(1 << order);
        std::vector<double> x, w;
        gauss_legendre01(pot_nu, x, w);
        Q.nu = pot_nu;
        for (int a = 0; a < pot_nu; ++a) {
            Q.du_u[a] = std::pow(x[a], pot_grade);
            Q.du_w[a] = w[a] * pot_grade * std::pow(x[a], pot_grade - 1);
        }
        gauss_legendre01(pot_nv, x, w);
        Q.nv = pot_nv;
        for (int b = 0; b < pot_nv; ++b) {
            Q.dv_v[b] = x[b];
            Q.dv_w[b] = w[b];
        }
        auto duffy_rule = [&](int nu, int nv, double *u, double *uw, double *v, double *vw) {
            std::vector<double> gx, gw;
            gauss_legendre01(nu, gx, gw);
            for (int a = 0; a < nu; ++a) {
                u[a] = std::pow(gx[a], pot_grade);
                uw[a] = gw[a] * pot_grade * std::pow(gx[a], pot_grade - 1);
            }
            gauss_legendre01(nv, gx, gw);
            for (int b = 0; b < nv; ++b) {
                v[b] = gx[b];
                vw[b] = gw[b];
            }
        };
        Q.lo_nu = std::max(2, pot_nu - 2);
        Q.lo_nv = std::max(2, pot_nv - 2);
        duffy_rule(Q.lo_nu, Q.lo_nv, Q.lo_u, Q.lo_uw, Q.lo_v, Q.lo_vw);
        Q.hi_nu = i2::kMaxDuffy;
        Q.hi_nv = i2::kMaxDuffy;
        duffy_rule(Q.hi_nu, Q.hi_nv, Q.hi_u, Q.hi_uw, Q.hi_v, Q.hi_vw);
        // tier 2b checks the 16 x 16 rule against 24 x 24 in the FP64 form.  The mixed form uses 20 x
        // 20: over the pairs where the choice changes the result (the 20,480-triangle sphere
        // jittered by 0.15 h: 1,322; a 1,280-triangle sphere jittered by 0.3 h: 845) the potential
        // stays within 1.1e-8 of the high-order answer (24 x 24: 4.6e-8 at most, p99 6e-10
        // against 8e-9), far below the FP32 bulk's 1e-7, for 21 % fewer FP64 points in the pass.
        Q.top_nu = mixed ? 20 : i2::kDuffyTop;
        Q.top_nv = Q.top_nu;
        duffy_rule(Q.top_nu, Q.top_nv, Q.top_u, Q.top_uw, Q.top_v, Q.top_vw);
        const int nself = self_points();
        gauss_legendre01(nself, x, w);
        Q.nself = nself;
        for (int k = 0; k < nself; ++k) {
            const double t = x[k];
            Q.sx[k] = t * t * (3.0 - 2.0 * t);
            Q.sw[k] = w[k] * 6.0 * t * (1.0 - t);
        }
        return Q;
    }
};

namespace {

struct ClassResult {
    int64_t n = 0;
    std::vector<int2> host_pairs;  // rows of the last host-side run (for output_results)
    DevBuf<double> raw4, J, P;
    DevBuf<int> level;
    DevBuf<int> maxlev;            // class-wide last refinement level of the last run (adjoint)
    DevBuf<int> counters;          // the run's 16 counters (i2_evaluator_run_stats)
    i2::RunConfig cfg;             // settings of the last run, adaptive-rule tolerance as applied (adjoint)
    double tier_tol = 0.0, top_tol = 0.0;  // tier bars of the last run (adjoint)
    i2_precision precision = I2_PRECISION_FP64;
    std::vector<double> errors;  // antisymmetry deltas (host)
};

struct Workspace {
    DevBuf<double> cur, fin_a, fin_b, sing, padj;
    DevBuf<float> ctx_e;
    DevBuf<int> stop, act_a, act_b, cnt, maxlev, hard_list, tier2_list, tier2b_list, pot_qcnt, fix_deep;
    DevBuf<i2::PotCellItem> pot_q_a, pot_q_b;
    DevBuf<long long> pot_fx;
    DevBuf<double> pot_ctx, pot_tri_a, pot_tri_b;
    DevBuf<double> fix_base, fix_part;
    DevBuf<int2> pairs;
};

} // namespace

struct i2_evaluator {
    const i2_mesh *mesh = nullptr;
    i2_integrator *integrator = nullptr;
    cudaStream_t stream = 0;
    ClassResult results[4];
    Workspace ws;
    int persistent_blocks = 0;
    // the mixed form runs an adjacent class's potential stages on `side`, beside its level chain
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~i2_evaluator()
    {
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
    }
};

// ------------------------------------------------------------------ pair lists (O(N))
namespace {

void build_pair_lists(i2_mesh &m, double near_factor)
{
    const int nc = m.nc(), nv = m.nv();
    for (auto &l : m.lists) l.clear();
    // vertex -> incident cells (CSR)
    std::vector<int> deg(nv + 1, 0);
    for (int v : m.C) deg[v + 1]++;
    for (int k = 0; k < nv; ++k) deg[k + 1] += deg[k];
    std::vector<int> inc(m.C.size()), fill(deg.begin(), deg.end() - 1);
    for (int c = 0; c < nc; ++c)
        for (int d = 0; d < 3; ++d) inc[fill[m.C[3 * c + d]]++] = c;
    // shared-vertex counts of the touching pairs of each cell
    std::vector<int> mark(nc, -1), shared(nc, 0), touched;
    for (int i = 0; i < nc; ++i) {
        touched.clear();
        for (int d = 0; d < 3; ++d) {
            const int v = m.C[3 * i + d];
            for (int q = deg[v]; q < deg[v + 1]; ++q) {
                const int j = inc[q];
                if (j <= i) continue;
                if (mark[j] != i) {
                    mark[j] = i;
                    shared[j] = 0;
                    touched.push_back(j);
                }
                shared[j]++;
            }
        }
        std::sort(touched.begin(), touched.end());
        for (int j : touched) {
            if (shared[j] == 1) { m.lists[I2_SIMPLE_NEIGHBORS].push_back(i); m.lists[I2_SIMPLE_NEIGHBORS].push_back(j); }
            else if (shared[j] == 2) { m.lists[I2_ATTACHED_NEIGHBORS].push_back(i); m.lists[I2_ATTACHED_NEIGHBORS].push_back(j); }
        }
        m.lists[I2_SELF].push_back(i);
        m.lists[I2_SELF].push_back(i);
    }
    // disjoint pairs: every pair (reference semantics) or centroid distance < near_factor x mean edge
    auto touching = [&](int i, int j) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                if (m.C[3 * i + a] == m.C[3 * j + b]) return true;
        return false;
    };
    auto &far = m.lists[I2_NOT_NEIGHBORS];
    if (near_factor <= 0) {
        I2_REQUIRE((long long)nc * nc <= 4000000000LL, I2_ERR_UNSUPPORTED, "all-pairs lists above 63k cells are not supported");
        for (int i = 0; i < nc; ++i)
            for (int j = i + 1; j < nc; ++j)
                if (!touching(i, j)) { far.push_back(i); far.push_back(j); }
        return;
    }
    const double r = near_factor * i2::mean_edge_length(m.V.data(), m.C.data(), nc);
    if (!(r > 0.0)) return;
    const i2::NearGrid g = i2::near_grid(m.centres.data(), nc, r);
    const double r2 = g.r2;
    const double *lo = g.lo;
    const long long *dims = g.dims;
    auto key = [&](long long x, long long y, long long z) { return (x * dims[1] + y) * dims[2] + z; };
    std::unordered_map<long long, std::vector<int>> grid;
    grid.reserve(nc);
    std::vector<long long> cx(nc), cy(nc), cz(nc);
    for (int c = 0; c < nc; ++c) {
        cx[c] = std::min(dims[0] - 1, (long long)((m.centres[3 * c] - lo[0]) / r));
        cy[c] = std::min(dims[1] - 1, (long long)((m.centres[3 * c + 1] - lo[1]) / r));
        cz[c] = std::min(dims[2] - 1, (long long)((m.centres[3 * c + 2] - lo[2]) / r));
        grid[key(cx[c], cy[c], cz[c])].push_back(c);
    }
    std::vector<int> cand;
    for (int i = 0; i < nc; ++i) {
        cand.clear();
        for (long long dx = -1; dx <= 1; ++dx)
            for (long long dy = -1; dy <= 1; ++dy)
                for (long long dz = -1; dz <= 1; ++dz) {
                    const long long x = cx[i] + dx, y = cy[i] + dy, z = cz[i] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= dims[0] || y >= dims[1] || z >= dims[2]) continue;
                    auto it = grid.find(key(x, y, z));
                    if (it == grid.end()) continue;
                    for (int j : it->second)
                        if (j > i) cand.push_back(j);
                }
        std::sort(cand.begin(), cand.end());
        for (int j : cand) {
            const double *p = &m.centres[3 * i], *q = &m.centres[3 * j];
            const double d2 = (p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]);
            if (d2 < r2 && !touching(i, j)) { far.push_back(i); far.push_back(j); }
        }
    }
}

// the host copy of a class's list, fetched once from the device when the mesh was prepared
// there without one
const std::vector<int> &host_list(const i2_mesh &cm, int cls)
{
    i2_mesh &m = const_cast<i2_mesh &>(cm);
    if (!m.host_lists) {
        for (int c = 0; c < 4; ++c) {
            m.lists[c].resize(2 * (size_t)m.dlists.n[c]);
            if (m.dlists.n[c])
                I2_CHECK_CUDA(cudaMemcpy(m.lists[c].data(), m.dlists.rows[c].ptr, m.dlists.n[c] * sizeof(int2), cudaMemcpyDeviceToHost));
        }
        m.host_lists = true;
    }
    return m.lists[cls];
}

int64_t list_size(const i2_mesh &m, int cls) { return m.host_lists ? (int64_t)m.lists[cls].size() / 2 : m.dlists.n[cls]; }

// the device copy of the lists, uploaded once when the mesh was prepared on the host
void device_lists(const i2_mesh &cm)
{
    i2_mesh &m = const_cast<i2_mesh &>(cm);
    if (m.dlists_ok) return;
    for (int c = 0; c < 4; ++c) {
        const int64_t n = (int64_t)m.lists[c].size() / 2;
        m.dlists.rows[c].release();
        m.dlists.rows[c].reserve(std::max<int64_t>(n, 1));
        if (n) I2_CHECK_CUDA(cudaMemcpy(m.dlists.rows[c].ptr, m.lists[c].data(), n * sizeof(int2), cudaMemcpyHostToDevice));
        m.dlists.n[c] = n;
    }
    m.dlists_ok = true;
}

void host_cell_geometry(i2_mesh &m)
{
    const int nc = m.nc();
    m.normals.assign(3 * nc, 0.0);
    m.measures.assign(nc, 0.0);
    m.centres.assign(3 * nc, 0.0);
    for (int c = 0; c < nc; ++c) {
        const double *A = &m.V[3 * m.C[3 * c]], *B = &m.V[3 * m.C[3 * c + 1]], *Cc = &m.V[3 * m.C[3 * c + 2]];
        const double u[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]}, v[3] = {Cc[0] - A[0], Cc[1] - A[1], Cc[2] - A[2]};
        const double cr[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        const double inv = 1.0 / len;
        for (int d = 0; d < 3; ++d) {
            m.normals[3 * c + d] = cr[d] * inv;
            m.centres[3 * c + d] = 0.3333333333333333 * (A[d] + B[d] + Cc[d]);
        }
        m.measures[c] = len * 0.5;
    }
}

void upload_mesh(i2_mesh &m)
{
    m.dV.reserve(m.V.size());
    m.dC.reserve(m.C.size());
    m.dPanels.reserve(m.nc());
    I2_CHECK_CUDA(cudaMemcpy(m.dV.ptr, m.V.data(), m.V.size() * sizeof(double), cudaMemcpyHostToDevice));
    I2_CHECK_CUDA(cudaMemcpy(m.dC.ptr, m.C.data(), m.C.size() * sizeof(int), cudaMemcpyHostToDevice));
    m.dPanelsF.reserve(m.nc());
    i2::launch_prepare_panels(m.nc(), m.dV.ptr, m.dC.ptr, m.dPanels.ptr, 0);
    i2::launch_prepare_panels_f32(m.nc(), m.dV.ptr, m.dC.ptr, m.dPanelsF.ptr, 0);
    I2_CHECK_CUDA(cudaGetLastError());
    I2_CHECK_CUDA(cudaDeviceSynchronize());
    m.on_device = true;
}

i2::QuadTablesF tables_f32(const i2::QuadTables &Q)
{
    i2::QuadTablesF F;
    std::memset(&F, 0, sizeof F);
    F.npts = Q.npts;
    F.pow2p = Q.pow2p;
    for (int g = 0; g < Q.npts; ++g) {
        F.L1[g] = (float)Q.L1[g];
        F.L2[g] = (float)Q.L2[g];
        F.L3[g] = (float)Q.L3[g];
        F.w[g] = (float)Q.w[g];
    }
    F.nu = Q.nu;
    F.nv = Q.nv;
    F.lo_nu = Q.lo_nu;
    F.lo_nv = Q.lo_nv;
    F.hi_nu = Q.hi_nu;
    F.top_nu = Q.top_nu;
    F.top_nv = Q.top_nv;
    for (int k = 0; k < i2::kDuffyTop; ++k) {
        F.top_u[k] = (float)Q.top_u[k]; F.top_uw[k] = (float)Q.top_uw[k]; F.top_v[k] = (float)Q.top_v[k]; F.top_vw[k] = (float)Q.top_vw[k];
    }
    F.hi_nv = Q.hi_nv;
    for (int k = 0; k < i2::kMaxDuffy; ++k) {
        F.du_u[k] = (float)Q.du_u[k]; F.du_w[k] = (float)Q.du_w[k]; F.dv_v[k] = (float)Q.dv_v[k]; F.dv_w[k] = (float)Q.dv_w[k];
        F.lo_u[k] = (float)Q.lo_u[k]; F.lo_uw[k] = (float)Q.lo_uw[k]; F.lo_v[k] = (float)Q.lo_v[k]; F.lo_vw[k] = (float)Q.lo_vw[k];
        F.hi_u[k] = (float)Q.hi_u[k]; F.hi_uw[k] = (float)Q.hi_uw[k]; F.hi_v[k] = (float)Q.hi_v[k]; F.hi_vw[k] = (float)Q.hi_vw[k];
    }
    return F;
}

// agreement bar of the tiered potential rule (main vs check Duffy rule, then main vs 16 x 16):
// 2e-7 keeps the rule within 1e-6 of the converged potential on the 20,480-triangle jittered
// sphere (largest error 6.5e-7 common vertex, 8.9e-7 common edge) and stays above the FP32
// rounding of the mixed form's Duffy sums
double tier_tolerance(const i2::RunConfig &cfg) { return std::max(10.0 * cfg.hard_tol, 2e-7); }
// agreement bar of tier 2b (16 x 16 against 24 x 24, FP64 in both forms): a tenth of the tier bar,
// since two rules that agree only to the tier bar can share a bias of 1e-6 (a near-coplanar pair of
// the sigma 0.3 jittered sphere)
double top_tolerance(const i2::RunConfig &cfg, bool) { return tier_tolerance(cfg) / 10.0; }
// relative tolerance of the adaptive potential rule: in the mixed form the FP64 rule stops at
// 2e-8, whatever tighter value the integrator holds (the FP32 bulk's own rounding is a few 1e-7).
// Over every common-edge pair and 60,000 common-vertex pairs of the 20,480-triangle jittered
// sphere, 2e-8 stays within 1.6e-8 of the 1e-8 result with 17-20 % fewer cells; looser values let
// the rule's local acceptance test pass cells that are off: 3e-8 gave 4.7e-7 on two common-edge
// pairs, 1e-7 gave 4.2e-6 on one.
constexpr double kMixedAdaptiveTol = 2e-8;
double adaptive_tolerance(const i2::RunConfig &cfg, bool mixed)
{
    return mixed && cfg.hard_tol > 0 ? std::max(cfg.hard_tol, kMixedAdaptiveTol) : cfg.hard_tol;
}

// cells per depth list of the adaptive potential (24 bytes each): every hard pair seeds 4 cells
// at depth 1; deeper lists hold a few tens of thousands of cells on the meshes measured (C2: at
// most 27,516).  Capped at 2^26 cells (1.5 GB per list).
size_t pot_queue_capacity(int64_t n) { return (size_t)std::min<int64_t>(std::max<int64_t>(4 * n, 1 << 18), 1 << 26); }
// caches of the adaptive potential, sized to the class (hard pairs are a small fraction; entries
// past the caps are recomputed): hard-pair set-ups, and parent-cell triangles per depth list
int pot_ctx_capacity(int64_t n)
{
    return (int)std::min<int64_t>(std::min<int64_t>(n, (int64_t)pot_queue_capacity(n) / 4), std::max<int64_t>(4096, n / 16));
}
int pot_tri_capacity(int64_t n) { return (int)std::min<int64_t>((int64_t)pot_queue_capacity(n) / 4, std::max<int64_t>(16384, n / 4)); }

i2_pair_class checked_class(int cls)
{
    I2_REQUIRE(cls >= 0 && cls <= 3, I2_ERR_INVALID_ARGUMENT, "pair class must be 0..3");
    return (i2_pair_class)cls;
}

// enqueue one class on the evaluator's stream; results land in the evaluator's buffers (or
// the caller's device buffers when given)
void run_class_device(i2_evaluator *ev, int cls, const int2 *d_pairs, int64_t n, double *out_raw, double *out_J,
                      double *out_P)
{
    I2_REQUIRE(ev->mesh->prepared, I2_ERR_STATE, "mesh not prepared");
    if (!ev->mesh->on_device) upload_mesh(const_cast<i2_mesh &>(*ev->mesh));
    const i2_mesh &m = *ev->mesh;
    I2_REQUIRE(n >= 0 && n < (1LL << 31), I2_ERR_INVALID_ARGUMENT, "pair count out of range");
    ClassResult &R = ev->results[cls];
    R.n = n;
    R.errors.clear();
    R.host_pairs.clear();
    if (n == 0) return;
    if (!out_raw) { R.raw4.reserve(4 * n); out_raw = R.raw4.ptr; }
    if (!out_J) { R.J.reserve(3 * n); out_J = R.J.ptr; }
    if (!out_P) { R.P.reserve(n); out_P = R.P.ptr; }
    R.level.reserve(n);
    const bool mixed = ev->integrator->precision == I2_PRECISION_MIXED;
    i2::RunConfig cfg = ev->integrator->cfg;
    const double tier_tol = tier_tolerance(cfg), top_tol = top_tolerance(cfg, mixed);
    cfg.hard_tol = adaptive_tolerance(cfg, mixed);
    Workspace &W = ev->ws;
    const bool adaptive = cfg.mode != i2::kFixed && cls != I2_SELF;
    W.cur.reserve(5 * n);
    if (adaptive) {
        W.fin_a.reserve(5 * n);
        W.fin_b.reserve(5 * n);
        W.stop.reserve(n);
        W.act_a.reserve(n);
        W.act_b.reserve(n);
    }
    // the mixed form gathers its needle-cell pairs for the FP64 fix-up into act_a
    if (mixed) {
        W.act_a.reserve(n);
        W.fix_deep.reserve(i2::kFixDeepCap);
        W.fix_base.reserve(5 * i2::kFixDeepCap);
        W.fix_part.reserve(5 * i2::kFixDeepSlots * i2::kFixDeepCap);
    }
    W.cnt.reserve(16);
    W.maxlev.reserve(1);
    if (cls == I2_SIMPLE_NEIGHBORS || cls == I2_ATTACHED_NEIGHBORS) {
        W.sing.reserve(4 * n);
        W.padj.reserve(n);
        W.hard_list.reserve(n);
        W.tier2_list.reserve(n);
        W.tier2b_list.reserve(n);
        W.pot_q_a.reserve(pot_queue_capacity(n));
        W.pot_q_b.reserve(pot_queue_capacity(n));
        W.pot_qcnt.reserve(16);
        W.pot_fx.reserve(n);
        W.pot_ctx.reserve((size_t)i2::kPotCtxDoubles * pot_ctx_capacity(n));
        W.pot_tri_a.reserve(9 * (size_t)pot_tri_capacity(n));
        W.pot_tri_b.reserve(9 * (size_t)pot_tri_capacity(n));
        if (ev->integrator->precision == I2_PRECISION_MIXED) W.ctx_e.reserve((size_t)i2::kPairCtxFloats * n);
    }
    // the run's counters (layout: kCnt* in i2_engine.h)
    I2_CHECK_CUDA(cudaMemsetAsync(W.cnt.ptr, 0, 16 * sizeof(int), ev->stream));
    I2_CHECK_CUDA(cudaMemsetAsync(W.maxlev.ptr, 0, sizeof(int), ev->stream));
    i2::ClassArgs A;
    A.n = (int)n;
    A.pairs = d_pairs;
    A.cells = reinterpret_cast<const int3 *>(m.dC.ptr);
    A.panels = m.dPanels.ptr;
    A.panels_f = m.dPanelsF.ptr;
    A.ctx_e = W.ctx_e.ptr;
    A.cur = W.cur.ptr;
    A.fin_a = W.fin_a.ptr;
    A.fin_b = W.fin_b.ptr;
    A.stop = W.stop.ptr;
    A.act_a = W.act_a.ptr;
    A.act_b = W.act_b.ptr;
    A.cnt = W.cnt.ptr;
    A.maxlev = W.maxlev.ptr;
    A.sing = W.sing.ptr;
    A.padj = W.padj.ptr;
    if (mixed) {
        A.fix_deep = W.fix_deep.ptr;
        A.fix_base = W.fix_base.ptr;
        A.fix_part = W.fix_part.ptr;
        A.fix_cap = i2::kFixDeepCap;
    }
    A.pot_off = cfg.potential ? 0 : 1;
    if ((cls == I2_SIMPLE_NEIGHBORS || cls == I2_ATTACHED_NEIGHBORS) && cfg.hard_tol > 0 && cfg.potential) {
        A.hard_list = W.hard_list.ptr;
        A.hard_cnt = W.cnt.ptr + i2::kCntHard;
        A.hard_overflow = W.cnt.ptr + i2::kCntOverflow;
        A.tier2_list = W.tier2_list.ptr;
        A.tier2b_list = W.tier2b_list.ptr;
        A.pot_q_a = W.pot_q_a.ptr;
        A.pot_q_b = W.pot_q_b.ptr;
        A.pot_qcap = (int)pot_queue_capacity(n);
        A.pot_qcnt = W.pot_qcnt.ptr;
        A.pot_fx = W.pot_fx.ptr;
        A.pot_ctx = W.pot_ctx.ptr;
        A.pot_ctx_cap = pot_ctx_capacity(n);
        A.pot_tri_a = W.pot_tri_a.ptr;
        A.pot_tri_b = W.pot_tri_b.ptr;
        A.pot_tri_cap = pot_tri_capacity(n);
        A.tier2_cnt = W.cnt.ptr + i2::kCntTier2;
        A.tier_tol = tier_tol;
        A.top_tol = top_tol;
    }
    A.raw4 = out_raw;
    A.J3 = out_J;
    A.P = out_P;
    A.level_out = R.level.ptr;
    if (ev->persistent_blocks == 0) {
        int dev = 0, sms = 0;
        I2_CHECK_CUDA(cudaGetDevice(&dev));
        I2_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        ev->persistent_blocks = std::max(1, sms) * 8;
    }
    const i2::QuadTables Q = ev->integrator->tables();
    if (ev->integrator->precision == I2_PRECISION_MIXED) {
        const i2::QuadTablesF Qf = tables_f32(Q);
        if (!ev->side) {
            I2_CHECK_CUDA(cudaStreamCreateWithFlags(&ev->side, cudaStreamNonBlocking));
            I2_CHECK_CUDA(cudaEventCreateWithFlags(&ev->fork, cudaEventDisableTiming));
            I2_CHECK_CUDA(cudaEventCreateWithFlags(&ev->join, cudaEventDisableTiming));
        }
        i2::launch_class_mixed(cls, A, Q, Qf, cfg, ev->persistent_blocks, ev->stream, i2::SideStream{ev->side, ev->fork, ev->join});
    } else {
        i2::launch_class_fp64(cls, A, Q, cfg, ev->persistent_blocks, ev->stream);
    }
    I2_CHECK_CUDA(cudaGetLastError());
    if (cls == I2_SELF) I2_CHECK_CUDA(cudaMemsetAsync(R.level.ptr, 0xff, n * sizeof(int), ev->stream));
    R.maxlev.reserve(1);
    I2_CHECK_CUDA(cudaMemcpyAsync(R.maxlev.ptr, W.maxlev.ptr, sizeof(int), cudaMemcpyDeviceToDevice, ev->stream));
    R.counters.reserve(16);
    I2_CHECK_CUDA(cudaMemcpyAsync(R.counters.ptr, W.cnt.ptr, 16 * sizeof(int), cudaMemcpyDeviceToDevice, ev->stream));
    R.cfg = cfg;
    R.tier_tol = tier_tol;
    R.top_tol = top_tol;
    R.precision = (i2_precision)ev->integrator->precision;
    // keep the evaluator's copies coherent when the caller supplied output buffers
    if (out_raw != R.raw4.ptr) { R.raw4.reserve(4 * n); I2_CHECK_CUDA(cudaMemcpyAsync(R.raw4.ptr, out_raw, 4 * n * sizeof(double), cudaMemcpyDeviceToDevice, ev->stream)); }
    if (out_J != R.J.ptr) { R.J.reserve(3 * n); I2_CHECK_CUDA(cudaMemcpyAsync(R.J.ptr, out_J, 3 * n * sizeof(double), cudaMemcpyDeviceToDevice, ev->stream)); }
    if (out_P != R.P.ptr) { R.P.reserve(n); I2_CHECK_CUDA(cudaMemcpyAsync(R.P.ptr, out_P, n * sizeof(double), cudaMemcpyDeviceToDevice, ev->stream)); }
}

void run_class_host(i2_evaluator *ev, int cls, const int32_t *rows, int64_t n, int stride)
{
    const int nc = ev->mesh->nc();
    std::vector<int2> pairs(n);
    for (int64_t k = 0; k < n; ++k) {
        const int i = rows[stride * k], j = rows[stride * k + 1];
        I2_REQUIRE(i >= 0 && i < nc && j >= 0 && j < nc, I2_ERR_INVALID_ARGUMENT, "pair index outside the mesh");
        pairs[k] = make_int2(i, j);
    }
    Workspace &W = ev->ws;
    W.pairs.reserve(std::max<int64_t>(n, 1));
    if (n) I2_CHECK_CUDA(cudaMemcpyAsync(W.pairs.ptr, pairs.data(), n * sizeof(int2), cudaMemcpyHostToDevice, ev->stream));
    run_class_device(ev, cls, W.pairs.ptr, n, nullptr, nullptr, nullptr);
    I2_CHECK_CUDA(cudaStreamSynchronize(ev->stream));
    ev->results[cls].host_pairs.swap(pairs);
}

} // namespace


// ------------------------------------------------------------------ batched form
namespace {

struct BatchSegment {
    const i2_mesh *mesh = nullptr;
    int cls = 0;
    int64_t n = 0;
    DevBuf<int2> pairs;
    DevBuf<double> raw4, J, P, cur, fin_a, fin_b, sing, padj;
    DevBuf<int> stop, act_a, act_b, cnt, maxlev, hard_list, tier2_list, tier2b_list, level, pot_qcnt, fix_deep;
    DevBuf<double> fix_base, fix_part;
    DevBuf<i2::PotCellItem> pot_q_a, pot_q_b;
    DevBuf<long long> pot_fx;
    DevBuf<double> pot_ctx, pot_tri_a, pot_tri_b;
    DevBuf<float> ctx_e;
    i2::ClassArgs args;
};

} // namespace

struct i2_batch {
    i2::RunConfig cfg;
    i2::QuadTables Q;
    i2::QuadTablesF Qf;
    std::vector<std::unique_ptr<BatchSegment>> segs;
    DevBuf<i2::BatchSeg> d_segs;
    i2::BatchTotals totals;
    bool dirty = true;
    cudaStream_t stream = 0;
    int threads = 256, blocks_per_sm = 0, g_cap = 32, variant = 0, sms = 0;
    cudaGraphExec_t graph = nullptr;
    bool graph_tried = false, graph_ok = false, last_graph = false;
    // the potential stages run on `side`, forked from and joined to the run's stream
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~i2_batch()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
    }
};

namespace {

void batch_prepare(i2_batch *b)
{
    if (!b->dirty) return;
    if (b->sms == 0) {
        int dev = 0;
        I2_CHECK_CUDA(cudaGetDevice(&dev));
        I2_CHECK_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
    }
    std::vector<i2::BatchSeg> hs;
    b->totals = i2::BatchTotals{};
    for (auto &sp : b->segs) {
        hs.push_back(i2::BatchSeg{sp->args, sp->cls});
        if (sp->n == 0) continue;
        if (sp->cls == I2_SELF) b->totals.self_pairs += sp->n;
        else {
            b->totals.present[sp->cls] = true;
            if (sp->cls != I2_NOT_NEIGHBORS) {
                b->totals.adjacent_pairs += sp->n;
                b->totals.hard_lists = b->totals.hard_lists || sp->args.hard_list != nullptr;
            }
            if (sp->args.act_a) b->totals.fixup_pairs += sp->n;
        }
    }
    b->d_segs.reserve(std::max<size_t>(hs.size(), 1));
    if (!hs.empty()) I2_CHECK_CUDA(cudaMemcpy(b->d_segs.ptr, hs.data(), hs.size() * sizeof(i2::BatchSeg), cudaMemcpyHostToDevice));
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->graph_tried = false;
    b->dirty = false;
}

// the whole batch on a stream: counter resets and closed forms, the cooperative level sweep (it
// runs alone: a cooperative grid is one resident wave), then two branches that share no data --
// the needle fix-up on `s` and the potential stages on the side stream, which fill the SMs the
// fix-up's few blocks leave idle -- joined back to `s`
void batch_enqueue(i2_batch *b, cudaStream_t s, int threads, int bps, int gcap, int variant)
{
    const int persistent = std::max(1, b->sms) * 8;
    const int nseg = (int)b->segs.size();
    if (nseg == 0) return;
    if (!b->side) {
        I2_CHECK_CUDA(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
        I2_CHECK_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
        I2_CHECK_CUDA(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming));
    }
    i2::RunConfig cfg = b->cfg;
    cfg.hard_tol = adaptive_tolerance(cfg, true);  // the batched form is mixed precision
    i2::launch_batch_singular(b->d_segs.ptr, nseg, b->totals, b->Qf, s);
    I2_REQUIRE(i2::batch_max_blocks_per_sm(threads, variant) > 0, I2_ERR_CUDA, "batch kernel cannot be resident with this block size");
    I2_CHECK_CUDA(i2::launch_batch_levels(b->d_segs.ptr, nseg, b->totals.present, b->Qf, b->cfg, b->sms, bps, threads, gcap, variant, s));
    I2_CHECK_CUDA(cudaEventRecord(b->fork, s));
    I2_CHECK_CUDA(cudaStreamWaitEvent(b->side, b->fork, 0));
    i2::launch_batch_potential(b->d_segs.ptr, nseg, b->totals, b->Q, b->Qf, cfg, persistent, b->side);
    i2::launch_batch_fixup(b->d_segs.ptr, nseg, b->totals, b->Q, b->cfg, persistent, s);
    I2_CHECK_CUDA(cudaEventRecord(b->join, b->side));
    I2_CHECK_CUDA(cudaStreamWaitEvent(s, b->join, 0));
    I2_CHECK_CUDA(cudaGetLastError());
}

} // namespace

void i2::set_last_error(const std::string &msg) { g_error = msg; }

// ------------------------------------------------------------------ C-ABI
extern "C" {

const char *i2_status_string(i2_status s)
{
    switch (s) {
    case I2_OK: return "ok";
    case I2_ERR_INVALID_ARGUMENT: return "invalid argument";
    case I2_ERR_CUDA: return "CUDA error";
    case I2_ERR_OUT_OF_MEMORY: return "out of memory";
    case I2_ERR_IO: return "I/O error";
    case I2_ERR_STATE: return "call out of order";
    case I2_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

const char *i2_last_error(void) { return g_error.c_str(); }
int32_t i2_version(void) { return 100; }

i2_status i2_mesh_create(i2_mesh_t **out)
{
    return guarded([&] {
        I2_REQUIRE(out, I2_ERR_INVALID_ARGUMENT, "null output pointer");
        *out = new i2_mesh();
    });
}

void i2_mesh_destroy(i2_mesh_t *mesh) { delete mesh; }

i2_status i2_mesh_load_file(i2_mesh_t *mesh, const char *path, double scale)
{
    return guarded([&] {
        I2_REQUIRE(mesh && path, I2_ERR_INVALID_ARGUMENT, "null argument");
        std::vector<double> V;
        std::vector<int> C;
        std::string err;
        if (!read_dat(path, scale, V, C, err)) throw Failure{I2_ERR_IO, err};
        mesh->V.swap(V);
        mesh->C.swap(C);
        mesh->prepared = false;
    });
}

i2_status i2_mesh_set_geometry(i2_mesh_t *mesh, const double *vertices, int32_t nv, const int32_t *cells, int32_t nc)
{
    return guarded([&] {
        I2_REQUIRE(mesh && (nv == 0 || vertices) && (nc == 0 || cells), I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(nv >= 0 && nc >= 0, I2_ERR_INVALID_ARGUMENT, "negative size");
        for (int64_t k = 0; k < 3LL * nc; ++k)
            I2_REQUIRE(cells[k] >= 0 && cells[k] < nv, I2_ERR_INVALID_ARGUMENT, "cell references a missing vertex");
        mesh->V.assign(vertices, vertices + 3LL * nv);
        mesh->C.assign(cells, cells + 3LL * nc);
        mesh->prepared = false;
    });
}

i2_status i2_mesh_prepare(i2_mesh_t *mesh, double near_factor)
{
    return guarded([&] {
        I2_REQUIRE(mesh, I2_ERR_INVALID_ARGUMENT, "null mesh");
        I2_REQUIRE(mesh->nc() > 0, I2_ERR_STATE, "mesh has no cells");
        host_cell_geometry(*mesh);
        for (int c = 0; c < mesh->nc(); ++c)
            I2_REQUIRE(mesh->measures[c] > 0.0 && std::isfinite(mesh->measures[c]), I2_ERR_INVALID_ARGUMENT,
                       "degenerate cell " + std::to_string(c));
        build_pair_lists(*mesh, near_factor);
        mesh->host_lists = true;
        mesh->dlists_ok = false;
        mesh->near_factor = near_factor;
        mesh->on_device = false;
        mesh->prepared = true;
    });
}

i2_status i2_mesh_prepare_device(i2_mesh_t *mesh, double near_factor, int32_t host_copy)
{
    return guarded([&] {
        I2_REQUIRE(mesh, I2_ERR_INVALID_ARGUMENT, "null mesh");
        I2_REQUIRE(mesh->nc() > 0, I2_ERR_STATE, "mesh has no cells");
        mesh->prepared = false;
        host_cell_geometry(*mesh);
        for (int c = 0; c < mesh->nc(); ++c)
            I2_REQUIRE(mesh->measures[c] > 0.0 && std::isfinite(mesh->measures[c]), I2_ERR_INVALID_ARGUMENT,
                       "degenerate cell " + std::to_string(c));
        upload_mesh(*mesh);
        mesh->on_device = true;
        for (auto &l : mesh->lists) std::vector<int>().swap(l);
        mesh->host_lists = false;
        mesh->dlists_ok = false;
        i2::build_pair_lists_device(mesh->V.data(), mesh->C.data(), mesh->centres.data(), mesh->nv(), mesh->nc(), mesh->dV.ptr,
                                    mesh->dC.ptr, near_factor, mesh->dlists, 0);
        mesh->dlists_ok = true;
        if (host_copy) host_list(*mesh, 0);
        mesh->near_factor = near_factor;
        mesh->prepared = true;
    });
}

i2_status i2_mesh_device_pairs(const i2_mesh_t *mesh, i2_pair_class cls, const int32_t **d_rows, int64_t *n)
{
    return guarded([&] {
        I2_REQUIRE(mesh && d_rows && n, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(mesh->prepared, I2_ERR_STATE, "mesh not prepared");
        const int c = checked_class(cls);
        device_lists(*mesh);
        *d_rows = reinterpret_cast<const int32_t *>(mesh->dlists.rows[c].ptr);
        *n = mesh->dlists.n[c];
    });
}

i2_status i2_mesh_sizes(const i2_mesh_t *mesh, int32_t *nv, int32_t *nc)
{
    return guarded([&] {
        I2_REQUIRE(mesh, I2_ERR_INVALID_ARGUMENT, "null mesh");
        if (nv) *nv = mesh->nv();
        if (nc) *nc = mesh->nc();
    });
}

i2_status i2_mesh_pair_count(const i2_mesh_t *mesh, i2_pair_class cls, int64_t *n)
{
    return guarded([&] {
        I2_REQUIRE(mesh && n, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(mesh->prepared, I2_ERR_STATE, "mesh not prepared");
        *n = list_size(*mesh, checked_class(cls));
    });
}

i2_status i2_mesh_copy_pairs(const i2_mesh_t *mesh, i2_pair_class cls, int32_t *rows, int64_t n)
{
    return guarded([&] {
        I2_REQUIRE(mesh && rows, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(mesh->prepared, I2_ERR_STATE, "mesh not prepared");
        const auto &l = host_list(*mesh, checked_class(cls));
        I2_REQUIRE(n == (int64_t)l.size() / 2, I2_ERR_INVALID_ARGUMENT, "row count does not match the list");
        for (int64_t k = 0; k < n; ++k) {
            rows[3 * k] = l[2 * k];
            rows[3 * k + 1] = l[2 * k + 1];
            rows[3 * k + 2] = (int32_t)k;
        }
    });
}

i2_status i2_mesh_copy_geometry(const i2_mesh_t *mesh, double *vertices, int32_t *cells)
{
    return guarded([&] {
        I2_REQUIRE(mesh, I2_ERR_INVALID_ARGUMENT, "null mesh");
        if (vertices) std::memcpy(vertices, mesh->V.data(), mesh->V.size() * sizeof(double));
        if (cells) std::memcpy(cells, mesh->C.data(), mesh->C.size() * sizeof(int32_t));
    });
}

i2_status i2_mesh_copy_cell_data(const i2_mesh_t *mesh, double *normals, double *measures, double *centres)
{
    return guarded([&] {
        I2_REQUIRE(mesh, I2_ERR_INVALID_ARGUMENT, "null mesh");
        I2_REQUIRE(mesh->prepared, I2_ERR_STATE, "mesh not prepared");
        if (normals) std::memcpy(normals, mesh->normals.data(), mesh->normals.size() * sizeof(double));
        if (measures) std::memcpy(measures, mesh->measures.data(), mesh->measures.size() * sizeof(double));
        if (centres) std::memcpy(centres, mesh->centres.data(), mesh->centres.size() * sizeof(double));
    });
}

i2_status i2_quadrature_builtin(int32_t npoints, double *coords, double *weights, int32_t *order)
{
    return guarded([&] {
        const Rule *r = builtin_rule(npoints);
        I2_REQUIRE(r, I2_ERR_INVALID_ARGUMENT, "no built-in rule with that many points (1,3,4,6,7,9,12,13)");
        if (coords) std::memcpy(coords, r->c.data(), r->c.size() * sizeof(double));
        if (weights) std::memcpy(weights, r->w.data(), r->w.size() * sizeof(double));
        if (order) *order = r->order;
    });
}

i2_status i2_integrator_create(const i2_mesh_t *mesh, const double *coords, const double *weights, int32_t npoints,
                               int32_t order, i2_integrator_t **out)
{
    return guarded([&] {
        I2_REQUIRE(mesh && coords && weights && out, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(npoints >= 1 && npoints <= i2::kMaxGauss, I2_ERR_INVALID_ARGUMENT, "1..16 quadrature points");
        I2_REQUIRE(order >= 1 && order <= 30, I2_ERR_INVALID_ARGUMENT, "order must be 1..30");
        auto it = std::make_unique<i2_integrator>();
        it->mesh = mesh;
        it->coords.assign(coords, coords + 2 * npoints);
        it->weights.assign(weights, weights + npoints);
        it->order = order;
        it->cfg.mode = i2::kAdaptiveCompat;  // the reference's default (NumericalIntegrator3d.cu:213)
        *out = it.release();
    });
}

void i2_integrator_destroy(i2_integrator_t *it) { delete it; }

i2_status i2_integrator_set_fixed_refinement_level(i2_integrator_t *it, int32_t level)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        I2_REQUIRE(level >= 0 && level <= 8, I2_ERR_INVALID_ARGUMENT, "fixed level must be 0..8");
        it->cfg.mode = i2::kFixed;
        it->cfg.level = level;
    });
}

i2_status i2_integrator_set_error_control(i2_integrator_t *it, i2_error_control mode, double rel_tol, int32_t max_level)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        I2_REQUIRE(mode >= 0 && mode <= 2, I2_ERR_INVALID_ARGUMENT, "unknown error-control mode");
        if (mode == I2_FIXED_REFINEMENT_LEVEL) {
            it->cfg.mode = i2::kFixed;
            return;
        }
        I2_REQUIRE(max_level >= 1 && max_level <= i2::kMaxLevel, I2_ERR_INVALID_ARGUMENT, "max level must be 1..5");
        I2_REQUIRE(mode != I2_RELATIVE_ERROR_CONTROL || (rel_tol > 0 && rel_tol < 1), I2_ERR_INVALID_ARGUMENT,
                   "relative tolerance must be in (0, 1)");
        it->cfg.mode = mode == I2_AUTOMATIC_ERROR_CONTROL ? i2::kAdaptiveCompat : i2::kAdaptiveRelative;
        it->cfg.tol = rel_tol;
        it->cfg.max_level = max_level;
    });
}

i2_status i2_integrator_get_error_control(const i2_integrator_t *it, i2_error_control *mode, int32_t *level)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        if (mode) *mode = (i2_error_control)it->cfg.mode;
        if (level) *level = it->cfg.mode == i2::kFixed ? it->cfg.level : it->cfg.max_level;
    });
}

i2_status i2_integrator_set_precision(i2_integrator_t *it, i2_precision precision)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        I2_REQUIRE(precision == I2_PRECISION_FP64 || precision == I2_PRECISION_MIXED, I2_ERR_INVALID_ARGUMENT,
                   "unknown precision");
        it->precision = precision;
    });
}

i2_status i2_integrator_set_potential_rule(i2_integrator_t *it, int32_t n_radial, int32_t n_angular, int32_t grading,
                                           int32_t n_self)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        I2_REQUIRE(n_radial >= 2 && n_radial <= i2::kMaxDuffy && n_angular >= 2 && n_angular <= i2::kMaxDuffy,
                   I2_ERR_INVALID_ARGUMENT, "Duffy rule sizes must be 2..16");
        I2_REQUIRE(grading >= 1 && grading <= 6, I2_ERR_INVALID_ARGUMENT, "grading must be 1..6");
        I2_REQUIRE(n_self == 0 || (n_self >= 2 && n_self <= i2::kMaxSelf), I2_ERR_INVALID_ARGUMENT, "self rule size must be 0 or 2..32");
        it->pot_nu = n_radial;
        it->pot_nv = n_angular;
        it->pot_grade = grading;
        it->pot_nself = n_self;
    });
}

i2_status i2_integrator_set_hard_pair_tolerance(i2_integrator_t *it, double rel_tol)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        I2_REQUIRE(rel_tol == 0.0 || (rel_tol >= 1e-13 && rel_tol < 1e-2), I2_ERR_INVALID_ARGUMENT,
                   "hard-pair tolerance must be 0 or in [1e-13, 1e-2)");
        it->cfg.hard_tol = rel_tol;
    });
}

i2_status i2_integrator_set_potential(i2_integrator_t *it, int32_t enabled)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        it->cfg.potential = enabled != 0;
    });
}

i2_status i2_integrator_set_self_convention(i2_integrator_t *it, int32_t sign)
{
    return guarded([&] {
        I2_REQUIRE(it, I2_ERR_INVALID_ARGUMENT, "null integrator");
        I2_REQUIRE(sign >= -1 && sign <= 1, I2_ERR_INVALID_ARGUMENT, "sign must be -1, 0 or 1");
        it->cfg.self_sign = sign;
    });
}

i2_status i2_evaluator_create(const i2_mesh_t *mesh, i2_integrator_t *it, i2_evaluator_t **out)
{
    return guarded([&] {
        I2_REQUIRE(mesh && it && out, I2_ERR_INVALID_ARGUMENT, "null argument");
        auto ev = std::make_unique<i2_evaluator>();
        ev->mesh = mesh;
        ev->integrator = it;
        *out = ev.release();
    });
}

void i2_evaluator_destroy(i2_evaluator_t *ev) { delete ev; }

i2_status i2_evaluator_set_stream(i2_evaluator_t *ev, void *stream)
{
    return guarded([&] {
        I2_REQUIRE(ev, I2_ERR_INVALID_ARGUMENT, "null evaluator");
        ev->stream = (cudaStream_t)stream;
    });
}

i2_status i2_evaluator_run_class(i2_evaluator_t *ev, i2_pair_class cls, const int32_t *rows, int64_t n, int32_t row_stride)
{
    return guarded([&] {
        I2_REQUIRE(ev && (n == 0 || rows), I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(row_stride == 2 || row_stride == 3, I2_ERR_INVALID_ARGUMENT, "row stride must be 2 or 3");
        run_class_host(ev, checked_class(cls), rows, n, row_stride);
    });
}

i2_status i2_evaluator_run_pairs(i2_evaluator_t *ev, const int32_t *simple, int64_t n_simple, const int32_t *attached,
                                 int64_t n_attached, const int32_t *not_neighbors, int64_t n_not)
{
    return guarded([&] {
        I2_REQUIRE(ev, I2_ERR_INVALID_ARGUMENT, "null evaluator");
        I2_REQUIRE((n_simple == 0 || simple) && (n_attached == 0 || attached) && (n_not == 0 || not_neighbors),
                   I2_ERR_INVALID_ARGUMENT, "null list");
        // the reference returns without work when all lists are empty (evaluator3d.cu:215-216)
        if (n_simple) run_class_host(ev, I2_SIMPLE_NEIGHBORS, simple, n_simple, 3);
        if (n_attached) run_class_host(ev, I2_ATTACHED_NEIGHBORS, attached, n_attached, 3);
        if (n_not) run_class_host(ev, I2_NOT_NEIGHBORS, not_neighbors, n_not, 3);
    });
}

i2_status i2_evaluator_run_all_pairs(i2_evaluator_t *ev, int32_t check_correctness)
{
    return guarded([&] {
        I2_REQUIRE(ev, I2_ERR_INVALID_ARGUMENT, "null evaluator");
        const i2_mesh &m = *ev->mesh;
        I2_REQUIRE(m.prepared, I2_ERR_STATE, "mesh not prepared");
        for (int cls = 0; cls < 4; ++cls) {
            const auto &l = host_list(m, cls);
            const int64_t u = (int64_t)l.size() / 2;
            std::vector<int32_t> rows;
            if (cls == I2_SELF) {
                rows.assign(l.begin(), l.end());
            } else {
                // rows 0..u-1 = (i, j), rows u..2u-1 = (j, i)  (kAddReversedPairs, evaluator3d.cu:22-31)
                rows.resize(4 * u);
                for (int64_t k = 0; k < u; ++k) {
                    rows[2 * k] = l[2 * k];
                    rows[2 * k + 1] = l[2 * k + 1];
                    rows[2 * (u + k)] = l[2 * k + 1];
                    rows[2 * (u + k) + 1] = l[2 * k];
                }
            }
            run_class_host(ev, cls, rows.data(), (int64_t)rows.size() / 2, 2);
            if (check_correctness && cls != I2_SELF && u > 0) {
                // kCalculateIntegrationError (evaluator3d.cu:45-57)
                std::vector<double> J(6 * u);
                I2_CHECK_CUDA(cudaMemcpy(J.data(), ev->results[cls].J.ptr, J.size() * sizeof(double), cudaMemcpyDeviceToHost));
                auto &err = ev->results[cls].errors;
                err.assign(2 * u, 0.0);
                for (int64_t k = 0; k < u; ++k) {
                    const double *a = &J[3 * k], *b = &J[3 * (u + k)];
                    const double s = std::fabs(a[0] + b[0]) + std::fabs(a[1] + b[1]) + std::fabs(a[2] + b[2]);
                    const double na = std::fabs(a[0]) + std::fabs(a[1]) + std::fabs(a[2]);
                    const double nb = std::fabs(b[0]) + std::fabs(b[1]) + std::fabs(b[2]);
                    err[k] = err[u + k] = s / std::max(na, nb);
                }
            }
        }
    });
}

i2_status i2_evaluator_run_class_device(i2_evaluator_t *ev, i2_pair_class cls, const int32_t *d_pairs, int64_t n,
                                        double *d_raw4, double *d_J, double *d_P)
{
    return guarded([&] {
        I2_REQUIRE(ev && (n == 0 || d_pairs), I2_ERR_INVALID_ARGUMENT, "null argument");
        run_class_device(ev, checked_class(cls), reinterpret_cast<const int2 *>(d_pairs), n, d_raw4, d_J, d_P);
    });
}

i2_status i2_evaluator_backward_class(i2_evaluator_t *ev, i2_pair_class cls, const int32_t *d_pairs, int64_t n,
                                      const double *d_gJ, const double *d_gP, double *d_gradV)
{
    return guarded([&] {
        I2_REQUIRE(ev && d_gradV && (n == 0 || d_pairs), I2_ERR_INVALID_ARGUMENT, "null argument");
        const int c = checked_class(cls);
        const ClassResult &R = ev->results[c];
        I2_REQUIRE(R.n == n, I2_ERR_STATE, "backward needs the forward run of this class with the same pairs just before");
        if (n == 0) return;
        const i2_mesh &m = *ev->mesh;
        I2_REQUIRE(m.on_device, I2_ERR_STATE, "mesh not on the device");
        // the settings and tier bars of the forward pass (run_class_device)
        i2::RunConfig cfg = R.cfg;
        I2_REQUIRE(cfg.potential, I2_ERR_UNSUPPORTED, "the adjoint needs the forward run with the potential (i2_integrator_set_potential)");
        const double tier_tol = R.tier_tol, top_tol = R.top_tol;
        if (ev->persistent_blocks == 0) {
            int dev = 0, sms = 0;
            I2_CHECK_CUDA(cudaGetDevice(&dev));
            I2_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            ev->persistent_blocks = std::max(1, sms) * 8;
        }
        i2::launch_adjoint(c, R.precision == I2_PRECISION_MIXED, reinterpret_cast<const int2 *>(d_pairs), (int)n,
                           reinterpret_cast<const int3 *>(m.dC.ptr), m.dV.ptr, R.level.ptr, R.maxlev.ptr, cfg, tier_tol, top_tol, d_gJ, d_gP,
                           d_gradV, ev->integrator->tables(), ev->persistent_blocks, ev->stream);
        I2_CHECK_CUDA(cudaGetLastError());
    });
}

i2_status i2_evaluator_synchronize(i2_evaluator_t *ev)
{
    return guarded([&] {
        I2_REQUIRE(ev, I2_ERR_INVALID_ARGUMENT, "null evaluator");
        I2_CHECK_CUDA(cudaStreamSynchronize(ev->stream));
    });
}

i2_status i2_evaluator_result_count(const i2_evaluator_t *ev, i2_pair_class cls, int64_t *n)
{
    return guarded([&] {
        I2_REQUIRE(ev && n, I2_ERR_INVALID_ARGUMENT, "null argument");
        *n = ev->results[checked_class(cls)].n;
    });
}

i2_status i2_evaluator_run_stats(const i2_evaluator_t *ev, i2_pair_class cls, int64_t *out, int32_t n)
{
    return guarded([&] {
        I2_REQUIRE(ev && out, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(n >= I2_RUN_STATS, I2_ERR_INVALID_ARGUMENT, "stats array too short");
        const ClassResult &R = ev->results[checked_class(cls)];
        for (int k = 0; k < I2_RUN_STATS; ++k) out[k] = 0;
        out[0] = R.n;
        if (R.n == 0 || !R.counters.ptr) return;
        int c[16], maxlev = 0;
        I2_CHECK_CUDA(cudaStreamSynchronize(ev->stream));
        I2_CHECK_CUDA(cudaMemcpy(c, R.counters.ptr, sizeof c, cudaMemcpyDeviceToHost));
        I2_CHECK_CUDA(cudaMemcpy(&maxlev, R.maxlev.ptr, sizeof maxlev, cudaMemcpyDeviceToHost));
        out[1] = c[i2::kCntTier2];
        out[2] = c[i2::kCntTier2b];
        out[3] = c[i2::kCntHard];
        out[4] = c[i2::kCntOverflow];
        out[5] = c[i2::kCntFixup];
        out[6] = maxlev;
        for (int L = 1; L <= 7; ++L) out[6 + L] = R.cfg.mode == i2::kFixed ? 0 : c[L];
        out[14] = std::min(c[i2::kCntFixDeep], i2::kFixDeepCap);
    });
}

i2_status i2_evaluator_copy_results(const i2_evaluator_t *ev, i2_pair_class cls, i2_channel channel, double *out, int64_t n)
{
    return guarded([&] {
        I2_REQUIRE(ev && (n == 0 || out), I2_ERR_INVALID_ARGUMENT, "null argument");
        const ClassResult &R = ev->results[checked_class(cls)];
        I2_REQUIRE(n == R.n, I2_ERR_INVALID_ARGUMENT, "count does not match the last run of this class");
        if (n == 0) return;
        I2_CHECK_CUDA(cudaStreamSynchronize(ev->stream));
        switch (channel) {
        case I2_CHANNEL_J: I2_CHECK_CUDA(cudaMemcpy(out, R.J.ptr, 3 * n * sizeof(double), cudaMemcpyDeviceToHost)); break;
        case I2_CHANNEL_P: I2_CHECK_CUDA(cudaMemcpy(out, R.P.ptr, n * sizeof(double), cudaMemcpyDeviceToHost)); break;
        case I2_CHANNEL_RAW: I2_CHECK_CUDA(cudaMemcpy(out, R.raw4.ptr, 4 * n * sizeof(double), cudaMemcpyDeviceToHost)); break;
        case I2_CHANNEL_ERROR:
            I2_REQUIRE(!R.errors.empty(), I2_ERR_STATE, "no antisymmetry check was run for this class");
            std::memcpy(out, R.errors.data(), n * sizeof(double));
            break;
        case I2_CHANNEL_LEVEL: {
            std::vector<int> lv(n);
            I2_CHECK_CUDA(cudaMemcpy(lv.data(), R.level.ptr, n * sizeof(int), cudaMemcpyDeviceToHost));
            for (int64_t k = 0; k < n; ++k) out[k] = lv[k];
            break;
        }
        default: throw Failure{I2_ERR_INVALID_ARGUMENT, "unknown channel"};
        }
    });
}

i2_status i2_evaluator_output_results(const i2_evaluator_t *ev, i2_pair_class cls, i2_output_format format, const char *path)
{
    return guarded([&] {
        I2_REQUIRE(ev && path, I2_ERR_INVALID_ARGUMENT, "null argument");
        const int c = checked_class(cls);
        const ClassResult &R = ev->results[c];
        I2_REQUIRE(R.n > 0, I2_ERR_STATE, "no results for this class");
        std::vector<double> J(3 * R.n);
        I2_CHECK_CUDA(cudaStreamSynchronize(ev->stream));
        I2_CHECK_CUDA(cudaMemcpy(J.data(), R.J.ptr, J.size() * sizeof(double), cudaMemcpyDeviceToHost));
        I2_REQUIRE((int64_t)R.host_pairs.size() == R.n, I2_ERR_STATE, "the last run of this class came from device rows");
        const std::vector<int2> &pairs = R.host_pairs;
        std::ofstream f(path);
        if (!f.is_open()) throw Failure{I2_ERR_IO, std::string("cannot open ") + path};
        if (format == I2_CSV_FULL_PRECISION) f << std::setprecision(17);
        const bool errors = !R.errors.empty();
        if (format != I2_PLAIN_TEXT) {
            f << "\"TaskI\";\"TaskJ\";\"IntegralX\";\"IntegralY\";\"IntegralZ\"";
            if (errors) f << ";\"Error\"";
            f << "\n";
        }
        for (int64_t k = 0; k < R.n; ++k) {
            if (format == I2_PLAIN_TEXT) {
                f << "(" << pairs[k].x << ", " << pairs[k].y << "): [" << J[3 * k] << ", " << J[3 * k + 1] << ", " << J[3 * k + 2] << "]";
                if (errors) f << ", error = " << R.errors[k];
            } else {
                f << pairs[k].x << ";" << pairs[k].y << ";" << J[3 * k] << ";" << J[3 * k + 1] << ";" << J[3 * k + 2];
                if (errors) f << ";" << R.errors[k];
            }
            f << "\n";
        }
    });
}

i2_status i2_batch_create(const i2_integrator_t *settings, i2_batch_t **out)
{
    return guarded([&] {
        I2_REQUIRE(settings && out, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(settings->cfg.potential, I2_ERR_UNSUPPORTED, "the batched form computes the potential (i2_integrator_set_potential)");
        auto b = std::make_unique<i2_batch>();
        b->cfg = settings->cfg;
        b->Q = settings->tables(true);  // the batched form is mixed precision
        b->Qf = tables_f32(b->Q);
        *out = b.release();
    });
}

void i2_batch_destroy(i2_batch_t *batch) { delete batch; }

i2_status i2_batch_set_stream(i2_batch_t *batch, void *stream)
{
    return guarded([&] {
        I2_REQUIRE(batch, I2_ERR_INVALID_ARGUMENT, "null batch");
        batch->stream = (cudaStream_t)stream;
        if (batch->graph) {
            cudaGraphExecDestroy(batch->graph);
            batch->graph = nullptr;
        }
        batch->graph_tried = false;
    });
}

i2_status i2_batch_add(i2_batch_t *batch, const i2_mesh_t *mesh, i2_pair_class cls, const int32_t *rows, int64_t n,
                       int32_t row_stride, int32_t *segment)
{
    return guarded([&] {
        I2_REQUIRE(batch && mesh && (n == 0 || rows), I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(row_stride == 2 || row_stride == 3, I2_ERR_INVALID_ARGUMENT, "row stride must be 2 or 3");
        I2_REQUIRE(mesh->prepared, I2_ERR_STATE, "mesh not prepared");
        I2_REQUIRE(n >= 0 && n < (1LL << 31), I2_ERR_INVALID_ARGUMENT, "pair count out of range");
        const int c = checked_class(cls);
        if (!mesh->on_device) upload_mesh(const_cast<i2_mesh &>(*mesh));
        const int nc = mesh->nc();
        std::vector<int2> pr(n);
        for (int64_t k = 0; k < n; ++k) {
            const int i = rows[row_stride * k], j = rows[row_stride * k + 1];
            I2_REQUIRE(i >= 0 && i < nc && j >= 0 && j < nc, I2_ERR_INVALID_ARGUMENT, "pair index outside the mesh");
            pr[k] = make_int2(i, j);
        }
        auto sp = std::make_unique<BatchSegment>();
        sp->mesh = mesh;
        sp->cls = c;
        sp->n = n;
        const size_t m = std::max<int64_t>(n, 1);
        sp->pairs.reserve(m);
        if (n) I2_CHECK_CUDA(cudaMemcpy(sp->pairs.ptr, pr.data(), n * sizeof(int2), cudaMemcpyHostToDevice));
        sp->raw4.reserve(4 * m); sp->J.reserve(3 * m); sp->P.reserve(m); sp->level.reserve(m);
        sp->cur.reserve(5 * m); sp->fin_a.reserve(5 * m); sp->fin_b.reserve(5 * m);
        sp->stop.reserve(m); sp->act_a.reserve(m); sp->act_b.reserve(m);
        sp->cnt.reserve(16); sp->maxlev.reserve(1);
        if (c != I2_SELF && n > 0) {
            // deep FP64 fix-up pairs of this segment (at most the segment's pairs)
            const int cap = (int)std::min<int64_t>(n, i2::kFixDeepCap);
            sp->fix_deep.reserve(cap); sp->fix_base.reserve(5 * (size_t)cap); sp->fix_part.reserve(5 * (size_t)i2::kFixDeepSlots * cap);
        }
        const bool adj = c == I2_SIMPLE_NEIGHBORS || c == I2_ATTACHED_NEIGHBORS;
        if (adj) {
            sp->sing.reserve(4 * m); sp->padj.reserve(m); sp->hard_list.reserve(m); sp->tier2_list.reserve(m); sp->tier2b_list.reserve(m); sp->ctx_e.reserve((size_t)i2::kPairCtxFloats * m);
            sp->pot_q_a.reserve(pot_queue_capacity(m)); sp->pot_q_b.reserve(pot_queue_capacity(m)); sp->pot_qcnt.reserve(16); sp->pot_fx.reserve(m);
            sp->pot_ctx.reserve((size_t)i2::kPotCtxDoubles * pot_ctx_capacity(m));
            sp->pot_tri_a.reserve(9 * (size_t)pot_tri_capacity(m)); sp->pot_tri_b.reserve(9 * (size_t)pot_tri_capacity(m));
        }
        i2::ClassArgs &A = sp->args;
        A.n = (int)n;
        A.pairs = sp->pairs.ptr;
        A.cells = reinterpret_cast<const int3 *>(mesh->dC.ptr);
        A.panels = mesh->dPanels.ptr;
        A.panels_f = mesh->dPanelsF.ptr;
        A.ctx_e = sp->ctx_e.ptr;
        A.cur = sp->cur.ptr; A.fin_a = sp->fin_a.ptr; A.fin_b = sp->fin_b.ptr; A.stop = sp->stop.ptr;
        A.act_a = sp->act_a.ptr; A.act_b = sp->act_b.ptr; A.cnt = sp->cnt.ptr; A.maxlev = sp->maxlev.ptr;
        A.sing = sp->sing.ptr; A.padj = sp->padj.ptr;
        if (adj && batch->cfg.hard_tol > 0) {
            A.hard_list = sp->hard_list.ptr; A.hard_cnt = sp->cnt.ptr + i2::kCntHard; A.hard_overflow = sp->cnt.ptr + i2::kCntOverflow;
            A.tier2_list = sp->tier2_list.ptr; A.tier2_cnt = sp->cnt.ptr + i2::kCntTier2; A.tier2b_list = sp->tier2b_list.ptr;
            A.pot_q_a = sp->pot_q_a.ptr; A.pot_q_b = sp->pot_q_b.ptr; A.pot_qcap = (int)pot_queue_capacity(m);
            A.pot_qcnt = sp->pot_qcnt.ptr; A.pot_fx = sp->pot_fx.ptr;
            A.pot_ctx = sp->pot_ctx.ptr; A.pot_ctx_cap = pot_ctx_capacity(m);
            A.pot_tri_a = sp->pot_tri_a.ptr; A.pot_tri_b = sp->pot_tri_b.ptr; A.pot_tri_cap = pot_tri_capacity(m);
            A.tier_tol = tier_tolerance(batch->cfg);
            A.top_tol = top_tolerance(batch->cfg, true);
        }
        A.raw4 = sp->raw4.ptr; A.J3 = sp->J.ptr; A.P = sp->P.ptr; A.level_out = sp->level.ptr;
        if (sp->fix_deep.ptr) {
            A.fix_deep = sp->fix_deep.ptr; A.fix_base = sp->fix_base.ptr; A.fix_part = sp->fix_part.ptr;
            A.fix_cap = (int)sp->fix_deep.count;
        }
        if (segment) *segment = (int32_t)batch->segs.size();
        batch->segs.push_back(std::move(sp));
        batch->dirty = true;
    });
}

i2_status i2_batch_autotune(i2_batch_t *batch, int32_t *shape)
{
    return guarded([&] {
        I2_REQUIRE(batch, I2_ERR_INVALID_ARGUMENT, "null batch");
        batch_prepare(batch);
        cudaEvent_t e0, e1;
        I2_CHECK_CUDA(cudaEventCreate(&e0));
        I2_CHECK_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        int bt = batch->threads, bb = batch->blocks_per_sm, bg = batch->g_cap, bv = batch->variant;
        auto time_shape = [&](int threads, int bps, int gcap, int variant) {
            batch_enqueue(batch, batch->stream, threads, bps, gcap, variant);  // warm-up
            I2_CHECK_CUDA(cudaEventRecord(e0, batch->stream));
            batch_enqueue(batch, batch->stream, threads, bps, gcap, variant);
            I2_CHECK_CUDA(cudaEventRecord(e1, batch->stream));
            I2_CHECK_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            I2_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) { best = ms; bt = threads; bb = bps; bg = gcap; bv = variant; }
        };
        // the shared shape with one register variant for every class ...
        for (int u : {0, 1, 2}) {
            const int variant = 13 * u;  // digit u for each of the three classes
            for (int threads : {128, 256}) {
                const int maxb = i2::batch_max_blocks_per_sm(threads, variant);
                if (maxb <= 0) continue;
                for (int bps : {maxb, std::max(1, maxb / 2)})
                    for (int gcap : {8, 16, 32}) time_shape(threads, bps, gcap, variant);
            }
        }
        // ... then each class's variant in turn, the others held (a class's level kernel has its
        // own register footprint: the disjoint class's fits 80 registers, the vertex class's
        // spills there); blocks per SM at the new variants' limit
        for (int place : {1, 3, 9}) {
            const int base = bv;
            for (int u : {0, 1, 2}) {
                const int variant = base - ((base / place) % 3) * place + u * place;
                if (variant == base) continue;
                const int maxb = i2::batch_max_blocks_per_sm(bt, variant);
                if (maxb > 0) time_shape(bt, bb == i2::batch_max_blocks_per_sm(bt, base) ? maxb : std::min(bb, maxb), bg, variant);
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        batch->threads = bt;
        batch->blocks_per_sm = bb;
        batch->g_cap = bg;
        batch->variant = bv;
        if (batch->graph) { cudaGraphExecDestroy(batch->graph); batch->graph = nullptr; }
        batch->graph_tried = false;
        if (shape) { shape[0] = bt; shape[1] = bb; shape[2] = bg; shape[3] = bv; }
    });
}

i2_status i2_batch_run(i2_batch_t *batch)
{
    return guarded([&] {
        I2_REQUIRE(batch, I2_ERR_INVALID_ARGUMENT, "null batch");
        batch_prepare(batch);
        if (!batch->graph_tried) {
            batch->graph_tried = true;
            // capture the whole batch once; a stream that cannot capture it runs direct launches
            cudaStream_t cs = batch->stream;
            bool own = false;
            if (cs == 0) {
                I2_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
                own = true;
            }
            cudaGraph_t g = nullptr;
            bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                try {
                    batch_enqueue(batch, cs, batch->threads, batch->blocks_per_sm, batch->g_cap, batch->variant);
                } catch (const Failure &) {
                    ok = false;
                }
                const cudaError_t e = cudaStreamEndCapture(cs, &g);
                ok = ok && e == cudaSuccess && g;
            }
            if (ok) ok = cudaGraphInstantiate(&batch->graph, g, 0) == cudaSuccess;
            if (g) cudaGraphDestroy(g);
            if (own) cudaStreamDestroy(cs);
            cudaGetLastError();  // a refused capture leaves a sticky-free error code behind
            batch->graph_ok = ok;
            if (!ok && batch->graph) { cudaGraphExecDestroy(batch->graph); batch->graph = nullptr; }
        }
        if (batch->graph_ok) {
            I2_CHECK_CUDA(cudaGraphLaunch(batch->graph, batch->stream));
            batch->last_graph = true;
        } else {
            batch_enqueue(batch, batch->stream, batch->threads, batch->blocks_per_sm, batch->g_cap, batch->variant);
            batch->last_graph = false;
        }
    });
}

i2_status i2_batch_uses_graph(const i2_batch_t *batch, int32_t *uses_graph)
{
    return guarded([&] {
        I2_REQUIRE(batch && uses_graph, I2_ERR_INVALID_ARGUMENT, "null argument");
        *uses_graph = batch->last_graph ? 1 : 0;
    });
}

i2_status i2_batch_result_count(const i2_batch_t *batch, int32_t segment, int64_t *n)
{
    return guarded([&] {
        I2_REQUIRE(batch && n, I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(segment >= 0 && segment < (int)batch->segs.size(), I2_ERR_INVALID_ARGUMENT, "no such segment");
        *n = batch->segs[segment]->n;
    });
}

i2_status i2_batch_copy_results(const i2_batch_t *batch, int32_t segment, i2_channel channel, double *out, int64_t n)
{
    return guarded([&] {
        I2_REQUIRE(batch && (n == 0 || out), I2_ERR_INVALID_ARGUMENT, "null argument");
        I2_REQUIRE(segment >= 0 && segment < (int)batch->segs.size(), I2_ERR_INVALID_ARGUMENT, "no such segment");
        const BatchSegment &S = *batch->segs[segment];
        I2_REQUIRE(n == S.n, I2_ERR_INVALID_ARGUMENT, "count does not match the segment");
        if (n == 0) return;
        I2_CHECK_CUDA(cudaStreamSynchronize(batch->stream));
        if (channel == I2_CHANNEL_J) I2_CHECK_CUDA(cudaMemcpy(out, S.J.ptr, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
        else if (channel == I2_CHANNEL_P) I2_CHECK_CUDA(cudaMemcpy(out, S.P.ptr, n * sizeof(double), cudaMemcpyDeviceToHost));
        else if (channel == I2_CHANNEL_RAW) I2_CHECK_CUDA(cudaMemcpy(out, S.raw4.ptr, 4 * n * sizeof(double), cudaMemcpyDeviceToHost));
        else if (channel == I2_CHANNEL_LEVEL) {
            std::vector<int> lv(n);
            I2_CHECK_CUDA(cudaMemcpy(lv.data(), S.level.ptr, n * sizeof(int), cudaMemcpyDeviceToHost));
            for (int64_t k = 0; k < n; ++k) out[k] = S.cls == I2_SELF ? -1 : lv[k];
        } else throw Failure{I2_ERR_INVALID_ARGUMENT, "channel not available for batch segments"};
    });
}

} // extern "C"
