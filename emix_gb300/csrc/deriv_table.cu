// deriv_table.cu -- host-side factor tables of the compact first derivative.
//
// Each scheme of the reference is a tridiagonal system  a_i x_{i-1} + b_i x_i
// + c_i x_{i+1} = r_i  with an explicit right-hand-side stencil.  The
// reference re-runs the Thomas recurrence for every pencil, one divide per
// row (src/Schemes/derivCompact.cu:199-212, solver/derivada.f90:111-122).
// Here the recurrence runs once per (scheme, n, h) on the host and the
// kernels only do multiply-adds: the pivot 1/bet_i and the 1/h scale are
// folded into the right-hand-side coefficients.
//
// The coefficient tables restate the reference:
//   A    solver/derivada.f90:22-89 (rows), :104-109 (RHS)
//   B    src/MSVSingle/derivada_incomp.f90:148-190,209-214 (rows), :306-313 (RHS)
//   BPER src/MSVSingle/derivada_incomp.f90:192-206 (rows), :231-247 (RHS, cyclic)
//   C    src/Schemes/derivCompact.cu:90-99 (RHS), :162-190 (rows)
#include "common.cuh"

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace emix {

namespace {

struct RowDef {
    double a, b, c;      // tridiagonal row
    int kind;            // 0 interior, 1 closure low (f_0..f_3), 2 closure high (f_{n-1}..f_{n-4})
    double ars, brs;     // interior stencil
    double cc[4];        // closure stencil
};

void set_interior(RowDef &r, double a, double c, double ars, double brs) {
    r.a = a; r.b = 1.0; r.c = c; r.kind = 0; r.ars = ars; r.brs = brs;
    for (double &v : r.cc) v = 0.0;
}

void set_closure(RowDef &r, int kind, double a, double c, double c0, double c1, double c2, double c3) {
    r.a = a; r.b = 1.0; r.c = c; r.kind = kind; r.ars = 0.0; r.brs = 0.0;
    r.cc[0] = c0; r.cc[1] = c1; r.cc[2] = c2; r.cc[3] = c3;
}

int define_rows(int scheme, int n, std::vector<RowDef> &R) {
    R.assign(n, RowDef{});
    switch (scheme) {
    case EMIX_SCHEME_A: {
        const double ars = 3. / 4., ars1 = -17. / 6., brs1 = 3. / 2., crs1 = 1.5, d1 = -1. / 6.;
        for (int i = 1; i < n - 1; ++i) set_interior(R[i], 1. / 4., 1. / 4., ars, 0.0);
        set_closure(R[0], 1, 0.0, 3.0, ars1, brs1, crs1, d1);
        set_closure(R[n - 1], 2, 3.0, 0.0, -ars1, -brs1, -crs1, -d1);
        // rows 1 and n-2 are interior rows of the reference; written as
        // closures so that the kernels never read f_{-1} or f_{n}
        set_closure(R[1], 1, 1. / 4., 1. / 4., -ars, 0.0, ars, 0.0);
        set_closure(R[n - 2], 2, 1. / 4., 1. / 4., ars, 0.0, -ars, 0.0);
        return 0;
    }
    case EMIX_SCHEME_B: {
        const double ars = 7. / 9., brs = 1. / 36., ars1 = -2.5, brs1 = 2., crs1 = 0.5, ars2 = 0.75;
        for (int i = 2; i < n - 2; ++i) set_interior(R[i], 1.0 / 3.0, 1.0 / 3.0, ars, brs);
        set_closure(R[0], 1, 0.0, 2.0, ars1, brs1, crs1, 0.0);
        set_closure(R[1], 1, 0.25, 0.25, -ars2, 0.0, ars2, 0.0);
        set_closure(R[n - 2], 2, 0.25, 0.25, ars2, 0.0, -ars2, 0.0);
        set_closure(R[n - 1], 2, 2.0, 0.0, -ars1, -brs1, -crs1, 0.0);
        return 0;
    }
    case EMIX_SCHEME_BPER: {
        const double ars = 7. / 9., brs = 1. / 36.;
        for (int i = 0; i < n; ++i) set_interior(R[i], 1.0 / 3.0, 1.0 / 3.0, ars, brs);
        return 0;
    }
    case EMIX_SCHEME_C: {
        const double ars = 14.0 / (9.0 * 2.0), brs = 1.0 / (9.0 * 4.0);
        const double ars1 = -17.0 / 6.0, brs1 = 3.0 / 2.0, crs1 = 3.0 / 2.0, drs1 = -1.0 / 6.0;
        const double ars2 = -3.0 / 4.0, crs2 = 3.0 / 4.0;
        for (int i = 2; i < n - 2; ++i) set_interior(R[i], 1.0 / 3.0, 1.0 / 3.0, ars, brs);
        set_closure(R[0], 1, 0.0, 3.0, ars1, brs1, crs1, drs1);
        set_closure(R[1], 1, 1.0 / 4.0, 1.0 / 4.0, ars2, 0.0, crs2, 0.0);
        set_closure(R[n - 2], 2, 1.0 / 4.0, 1.0 / 4.0, -ars2, 0.0, -crs2, 0.0);
        set_closure(R[n - 1], 2, 3.0, 0.0, -ars1, -brs1, -crs1, -drs1);
        return 0;
    }
    default:
        return 1;
    }
}

} // namespace

namespace {

// the table of (sign/h) * A^{-1} B: sign = -1 gives -D, which is D^T for the
// cyclic scheme (A symmetric circulant, B antisymmetric circulant)
int build_table_signed(int scheme, int n, double h, double sign, DerivTable &t, DerivRow *rows,
                       double *clo, double *chi, double *u0, double *zz);

} // namespace

int build_deriv_table_host(int scheme, int n, double h, DerivTable &t, DerivRow *rows,
                           double *clo, double *chi, double *u0, double *zz) {
    if (n < 6 || n > kTableMaxN || !(h > 0.0)) return EMIX_ERR_ARG;
    return build_table_signed(scheme, n, h, 1.0, t, rows, clo, chi, u0, zz);
}

namespace {

int build_table_signed(int scheme, int n, double h, double sign, DerivTable &t, DerivRow *rows,
                       double *clo, double *chi, double *u0, double *zz) {
    std::vector<RowDef> R;
    if (define_rows(scheme, n, R)) return EMIX_ERR_ARG;
    const bool per = scheme == EMIX_SCHEME_BPER;
    const double s = sign / h;

    std::vector<double> bb(n), bet(n), gam(n, 0.0);
    for (int i = 0; i < n; ++i) bb[i] = R[i].b;
    double alpha = 0.0, beta = 0.0, gamma = 0.0;
    if (per) {  // Sherman-Morrison split of the cyclic matrix (derivada_incomp.f90:243-250)
        alpha = R[0].a;
        beta = R[n - 1].c;
        gamma = -R[0].b;
        bb[0] = R[0].b - gamma;
        bb[n - 1] = R[n - 1].b - alpha * beta / gamma;
    }
    bet[0] = bb[0];
    for (int i = 1; i < n; ++i) {
        gam[i] = R[i - 1].c / bet[i - 1];
        bet[i] = bb[i] - R[i].a * gam[i];
        if (bet[i] == 0.0 || !std::isfinite(bet[i])) return EMIX_ERR_ARG;
    }

    t.n = n;
    t.scheme = scheme;
    t.periodic = per ? 1 : 0;
    t.nlo = t.nhi = 0;
    for (int k = 0; k < kMaxClosure * 4; ++k) clo[k] = chi[k] = 0.0;
    for (int i = 0; i < n; ++i) {
        const double ib = 1.0 / bet[i];
        DerivRow &r = rows[i];
        r.A = s * R[i].ars * ib;
        r.B = s * R[i].brs * ib;
        r.m = i == 0 ? 0.0 : R[i].a * ib;
        r.g = i == n - 1 ? 0.0 : gam[i + 1];
        if (R[i].kind == 1) {
            if (i != t.nlo || t.nlo >= kMaxClosure) return EMIX_ERR_ARG;
            for (int q = 0; q < 4; ++q) clo[4 * t.nlo + q] = s * R[i].cc[q] * ib;
            ++t.nlo;
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        if (R[i].kind != 2) continue;
        const int k = n - 1 - i;
        if (k != t.nhi || t.nhi >= kMaxClosure) return EMIX_ERR_ARG;
        const double ib = 1.0 / bet[i];
        for (int q = 0; q < 4; ++q) chi[4 * t.nhi + q] = s * R[i].cc[q] * ib;
        ++t.nhi;
    }

    // the pencil kernels assume two explicit closure rows at each wall
    if (!per && (t.nlo != 2 || t.nhi != 2)) return EMIX_ERR_ARG;

    t.ku = 0; t.zlo = 0; t.zhi = n; t.sm1 = 0.0; t.sm2 = 0.0;
    if (per) {
        // zz = A'^{-1} (gamma, 0, ..., 0, alpha): same forward/backward sweep
        std::vector<double> w(n);
        w[0] = gamma / bet[0];
        for (int i = 1; i < n; ++i) {
            double ri = (i == n - 1) ? alpha : 0.0;
            w[i] = (ri - R[i].a * w[i - 1]) / bet[i];
        }
        zz[n - 1] = w[n - 1];
        for (int i = n - 2; i >= 0; --i) zz[i] = w[i] - gam[i + 1] * zz[i + 1];
        // y_0 = sum_k U0_k w_k with U0_k = prod_{j<k} (-gam_{j+1})
        double p = 1.0;
        int ku = 0;
        while (ku < n && std::fabs(p) > 1e-22) {
            u0[ku++] = p;
            if (ku < n) p *= -gam[ku];
        }
        t.ku = ku;
        t.sm1 = beta / gamma;
        t.sm2 = 1.0 / (1.0 + zz[0] + t.sm1 * zz[n - 1]);
        double zmax = 0.0;
        for (int i = 0; i < n; ++i) zmax = std::fmax(zmax, std::fabs(zz[i]));
        const double thr = 1e-22 * zmax;
        int zlo = 0;
        while (zlo < n && std::fabs(zz[zlo]) > thr) ++zlo;
        int zhi = n;
        while (zhi > 0 && std::fabs(zz[zhi - 1]) > thr) --zhi;
        if (zlo >= zhi) { zlo = n; zhi = n; }
        t.zlo = zlo;
        t.zhi = zhi;
    }
    return EMIX_OK;
}

struct TableKey {
    int dev, scheme, n;
    double h;
    bool operator<(const TableKey &o) const {
        return std::tie(dev, scheme, n, h) < std::tie(o.dev, o.scheme, o.n, o.h);
    }
};

std::mutex g_table_mu;
std::map<TableKey, DerivTable> g_tables;   // device buffers live until process exit

} // namespace

int get_table_signed(int scheme, int n, double h, double sign, DerivTable *out);

int get_deriv_table(int scheme, int n, double h, DerivTable *out) {
    if (!(h > 0.0)) return EMIX_ERR_ARG;
    return get_table_signed(scheme, n, h, 1.0, out);
}

int get_table_signed(int scheme, int n, double h, double sign, DerivTable *out) {
    int dev = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    TableKey key{dev, scheme, n, sign * h};
    std::lock_guard<std::mutex> lock(g_table_mu);
    auto it = g_tables.find(key);
    if (it != g_tables.end()) {
        *out = it->second;
        return EMIX_OK;
    }
    if (n < 6 || n > kTableMaxN) return EMIX_ERR_ARG;
    std::vector<DerivRow> rows(n);
    std::vector<double> clo(kMaxClosure * 4), chi(kMaxClosure * 4), u0(n, 0.0), zz(n, 0.0);
    DerivTable t{};
    int rc = build_table_signed(scheme, n, h, sign, t, rows.data(), clo.data(), chi.data(),
                                u0.data(), zz.data());
    if (rc) return rc;
    // the scaled form: k_i = A_i on stencil rows, 1 on the closure rows
    std::vector<double> kap(n), u0s(n, 0.0);
    std::vector<DerivRowU> urows(n);
    for (int i = 0; i < n; ++i) {
        const bool closure = !t.periodic && (i < t.nlo || i >= n - t.nhi);
        kap[i] = closure ? 1.0 : rows[i].A;
        if (kap[i] == 0.0 || !std::isfinite(kap[i])) return EMIX_ERR_ARG;
    }
    for (int i = 0; i < n; ++i) {
        const bool closure = !t.periodic && (i < t.nlo || i >= n - t.nhi);
        DerivRowU &u = urows[i];
        u.c = closure ? 0.0 : rows[i].B / rows[i].A;
        u.mu = i == 0 ? 0.0 : rows[i].m * (kap[i - 1] / kap[i]);
        u.gu = i == n - 1 ? 0.0 : rows[i].g * (kap[i + 1] / kap[i]);
        u.k = kap[i];
    }
    for (int k = 0; k < t.ku; ++k) u0s[k] = u0[k] * kap[k];
    t.sm1s = t.sm1 * kap[n - 1];
    // one allocation: rows | clo | chi | u0 | zz | urows | u0s
    const size_t nd = (size_t)4 * n + 8 * kMaxClosure + 2 * (size_t)n + 4 * (size_t)n + n;
    double *buf = nullptr;
    if (cudaMalloc(&buf, nd * sizeof(double)) != cudaSuccess) {
        set_last_message("cudaMalloc of a derivative table failed");
        return EMIX_ERR_ALLOC;
    }
    std::vector<double> host(nd);
    std::memcpy(host.data(), rows.data(), (size_t)n * sizeof(DerivRow));
    double *p = host.data() + 4 * (size_t)n;
    std::memcpy(p, clo.data(), 4 * kMaxClosure * sizeof(double));
    std::memcpy(p + 4 * kMaxClosure, chi.data(), 4 * kMaxClosure * sizeof(double));
    std::memcpy(p + 8 * kMaxClosure, u0.data(), (size_t)n * sizeof(double));
    std::memcpy(p + 8 * kMaxClosure + n, zz.data(), (size_t)n * sizeof(double));
    std::memcpy(p + 8 * kMaxClosure + 2 * n, urows.data(), (size_t)n * sizeof(DerivRowU));
    std::memcpy(p + 8 * kMaxClosure + 6 * n, u0s.data(), (size_t)n * sizeof(double));
    EMIX_CUDA_TRY(cudaMemcpy(buf, host.data(), nd * sizeof(double), cudaMemcpyHostToDevice));
    t.rows = reinterpret_cast<const DerivRow *>(buf);
    t.clo = buf + 4 * (size_t)n;
    t.chi = t.clo + 4 * kMaxClosure;
    t.u0 = t.chi + 4 * kMaxClosure;
    t.zz = t.u0 + n;
    t.urows = reinterpret_cast<const DerivRowU *>(t.zz + n);
    t.u0s = t.zz + 5 * (size_t)n;
    g_tables[key] = t;
    *out = t;
    return EMIX_OK;
}

// ---- PCR + Thomas tables ----------------------------------------------------

namespace {

struct PKey {
    int dev, scheme, n, steps;
    double h;
    bool operator<(const PKey &o) const {
        return std::tie(dev, scheme, n, steps, h) < std::tie(o.dev, o.scheme, o.n, o.steps, o.h);
    }
};

std::mutex g_p_mu;
std::map<PKey, PcrTable> g_p_tables;   // device buffers live until process exit

} // namespace

int get_pcr_table(int scheme, int n, double h, int steps, PcrTable *out) {
    if (!(h > 0.0) || steps < 1 || steps > kPcrMaxSteps || n < 6 || n > kPcrMaxN) return EMIX_ERR_ARG;
    int dev = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    PKey key{dev, scheme, n, steps, h};
    std::lock_guard<std::mutex> lock(g_p_mu);
    auto it = g_p_tables.find(key);
    if (it != g_p_tables.end()) {
        *out = it->second;
        return EMIX_OK;
    }
    std::vector<RowDef> R;
    if (define_rows(scheme, n, R)) return EMIX_ERR_ARG;
    const bool per = scheme == EMIX_SCHEME_BPER;
    PcrTable t{};
    t.n = n; t.steps = steps; t.periodic = per ? 1 : 0;
    // the non-cyclic matrix A' (the cyclic one with the Sherman-Morrison
    // corners folded into the diagonal, derivada_incomp.f90:243-250)
    std::vector<double> a(n), b(n), c(n);
    for (int i = 0; i < n; ++i) { a[i] = R[i].a; b[i] = R[i].b; c[i] = R[i].c; }
    double alpha = 0.0, beta = 0.0, gamma = 0.0;
    if (per) {
        alpha = R[0].a; beta = R[n - 1].c; gamma = -R[0].b;
        b[0] = R[0].b - gamma;
        b[n - 1] = R[n - 1].b - alpha * beta / gamma;
    }
    a[0] = 0.0;
    c[n - 1] = 0.0;
    // right-hand side, 1/h folded in
    std::vector<double> ra(n, 0.0), rb(n, 0.0), cl(4 * (size_t)n, 0.0);
    t.nlo = t.nhi = 0;
    for (int i = 0; i < n; ++i) {
        if (R[i].kind == 0) {
            ra[i] = R[i].ars / h;
            rb[i] = R[i].brs / h;
        } else {
            for (int q = 0; q < 4; ++q) cl[4 * i + q] = R[i].cc[q] / h;
            if (R[i].kind == 1) ++t.nlo; else ++t.nhi;
        }
    }
    // PCR on the matrix side
    std::vector<double> al((size_t)steps * n), ga((size_t)steps * n);
    for (int k = 0; k < steps; ++k) {
        const int hs = 1 << k;
        std::vector<double> a2(n), b2(n), c2(n);
        for (int i = 0; i < n; ++i) {
            const double am = i - hs >= 0 ? -a[i] / b[i - hs] : 0.0;
            const double gp = i + hs < n ? -c[i] / b[i + hs] : 0.0;
            al[(size_t)k * n + i] = am;
            ga[(size_t)k * n + i] = gp;
            a2[i] = i - hs >= 0 ? am * a[i - hs] : 0.0;
            c2[i] = i + hs < n ? gp * c[i + hs] : 0.0;
            b2[i] = b[i] + (i - hs >= 0 ? am * c[i - hs] : 0.0) + (i + hs < n ? gp * a[i + hs] : 0.0);
            if (b2[i] == 0.0 || !std::isfinite(b2[i])) return EMIX_ERR_ARG;
        }
        a = a2; b = b2; c = c2;
    }
    // Thomas factors of each subsystem (rows r, r + H, r + 2H, ...)
    const int H = 1 << steps;
    std::vector<double> ib(n), mt(n), gt(n);
    for (int r = 0; r < H && r < n; ++r) {
        double bet = 0.0;
        for (int i = r; i < n; i += H) {
            if (i == r) {
                bet = b[i];
                mt[i] = 0.0;
            } else {
                const double gam = c[i - H] / bet;
                bet = b[i] - a[i] * gam;
                mt[i] = a[i] / bet;
            }
            if (bet == 0.0 || !std::isfinite(bet)) return EMIX_ERR_ARG;
            ib[i] = 1.0 / bet;
            gt[i] = c[i] / bet;
        }
    }
    // cyclic correction: zz = A'^{-1} (gamma, 0, ..., 0, alpha) by plain Thomas
    std::vector<double> zz(n, 0.0);
    if (per) {
        std::vector<double> A0(n), B0(n), C0(n), w(n), bet(n), gam(n, 0.0);
        for (int i = 0; i < n; ++i) { A0[i] = R[i].a; B0[i] = R[i].b; C0[i] = R[i].c; }
        B0[0] = R[0].b - gamma;
        B0[n - 1] = R[n - 1].b - alpha * beta / gamma;
        bet[0] = B0[0];
        w[0] = gamma / bet[0];
        for (int i = 1; i < n; ++i) {
            gam[i] = C0[i - 1] / bet[i - 1];
            bet[i] = B0[i] - A0[i] * gam[i];
            const double ri = i == n - 1 ? alpha : 0.0;
            w[i] = (ri - A0[i] * w[i - 1]) / bet[i];
        }
        zz[n - 1] = w[n - 1];
        for (int i = n - 2; i >= 0; --i) zz[i] = w[i] - gam[i + 1] * zz[i + 1];
        t.sm1 = beta / gamma;
        t.sm2 = 1.0 / (1.0 + zz[0] + t.sm1 * zz[n - 1]);
    }
    // one allocation: ra | rb | cl | al | ga | ib | mt | gt | zz
    const size_t nd = (size_t)n * (2 + 4 + 2 * steps + 4);
    std::vector<double> host;
    host.reserve(nd);
    host.insert(host.end(), ra.begin(), ra.end());
    host.insert(host.end(), rb.begin(), rb.end());
    host.insert(host.end(), cl.begin(), cl.end());
    host.insert(host.end(), al.begin(), al.end());
    host.insert(host.end(), ga.begin(), ga.end());
    host.insert(host.end(), ib.begin(), ib.end());
    host.insert(host.end(), mt.begin(), mt.end());
    host.insert(host.end(), gt.begin(), gt.end());
    host.insert(host.end(), zz.begin(), zz.end());
    double *buf = nullptr;
    if (cudaMalloc(&buf, nd * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        set_last_message("cudaMalloc of a PCR table failed");
        return EMIX_ERR_ALLOC;
    }
    EMIX_CUDA_TRY(cudaMemcpy(buf, host.data(), nd * sizeof(double), cudaMemcpyHostToDevice));
    double *q = buf;
    t.ra = q; q += n;
    t.rb = q; q += n;
    t.cl = q; q += 4 * (size_t)n;
    t.al = q; q += (size_t)steps * n;
    t.ga = q; q += (size_t)steps * n;
    t.ib = q; q += n;
    t.mt = q; q += n;
    t.gt = q; q += n;
    t.zz = q;
    g_p_tables[key] = t;
    *out = t;
    return EMIX_OK;
}

// ---- transposed operator D^T = B^T A^{-T} (the adjoint's pencil solves) ----

namespace {

struct TKey {
    int dev, scheme, n;
    double h;
    bool operator<(const TKey &o) const {
        return std::tie(dev, scheme, n, h) < std::tie(o.dev, o.scheme, o.n, o.h);
    }
};

std::mutex g_t_mu;
std::map<TKey, DerivTTable> g_t_tables;

// A^T (sub-diagonal c_{i-1}, super-diagonal a_{i+1}) factored once; B^T as a
// band of 7 (offsets -3..3, the closure rows reach 3 away), 1/h folded in
int build_t_host(int scheme, int n, double h, std::vector<DerivTRow> &rows, std::vector<double> &bt) {
    std::vector<RowDef> R;
    if (define_rows(scheme, n, R)) return EMIX_ERR_ARG;
    const double s = 1.0 / h;
    rows.assign(n, DerivTRow{});
    std::vector<double> bet(n), gam(n + 1, 0.0);
    bet[0] = R[0].b;
    for (int i = 1; i < n; ++i) {
        gam[i] = R[i].a / bet[i - 1];                 // super-diagonal of A^T at row i-1
        bet[i] = R[i].b - R[i - 1].c * gam[i];        // sub-diagonal of A^T at row i: c_{i-1}
        if (bet[i] == 0.0 || !std::isfinite(bet[i])) return EMIX_ERR_ARG;
    }
    for (int i = 0; i < n; ++i) {
        const double ib = 1.0 / bet[i];
        rows[i].ib = ib;
        rows[i].m = i == 0 ? 0.0 : R[i - 1].c * ib;
        rows[i].g = i == n - 1 ? 0.0 : gam[i + 1];
    }
    // B as rows: B[i][j]; B^T[j][i - j + 3] = B[i][j]
    bt.assign((size_t)7 * n, 0.0);
    auto put = [&](int i, int j, double v) {
        const int k = i - j + 3;
        if (j < 0 || j >= n || k < 0 || k > 6) return false;
        bt[(size_t)7 * j + k] += s * v;
        return true;
    };
    for (int i = 0; i < n; ++i) {
        const RowDef &r = R[i];
        bool ok = true;
        if (r.kind == 0) {
            ok = ok && (r.ars == 0.0 || (put(i, i + 1, r.ars) && put(i, i - 1, -r.ars)));
            ok = ok && (r.brs == 0.0 || (put(i, i + 2, r.brs) && put(i, i - 2, -r.brs)));
        } else if (r.kind == 1) {
            for (int q = 0; q < 4; ++q) if (r.cc[q] != 0.0) ok = ok && put(i, q, r.cc[q]);
        } else {
            for (int q = 0; q < 4; ++q) if (r.cc[q] != 0.0) ok = ok && put(i, n - 1 - q, r.cc[q]);
        }
        if (!ok) return EMIX_ERR_ARG;
    }
    return EMIX_OK;
}

} // namespace

int get_deriv_t_table(int scheme, int n, double h, DerivTTable *out) {
    if (!(h > 0.0) || n < 6 || n > kTableMaxN) return EMIX_ERR_ARG;
    int dev = 0;
    EMIX_CUDA_TRY(cudaGetDevice(&dev));
    TKey key{dev, scheme, n, h};
    {
        std::lock_guard<std::mutex> lock(g_t_mu);
        auto it = g_t_tables.find(key);
        if (it != g_t_tables.end()) {
            *out = it->second;
            return EMIX_OK;
        }
    }
    DerivTTable t{};
    t.n = n;
    if (scheme == EMIX_SCHEME_BPER) {
        // cyclic scheme: D^T = -D, the forward kernels with -1/h
        t.periodic = 1;
        int rc = get_table_signed(scheme, n, h, -1.0, &t.neg);
        if (rc) return rc;
    } else {
        std::vector<DerivTRow> rows;
        std::vector<double> bt;
        int rc = build_t_host(scheme, n, h, rows, bt);
        if (rc) return rc;
        const size_t nd = (size_t)3 * n + bt.size();
        double *buf = nullptr;
        if (cudaMalloc(&buf, nd * sizeof(double)) != cudaSuccess) {
            set_last_message("cudaMalloc of a transposed derivative table failed");
            return EMIX_ERR_ALLOC;
        }
        std::vector<double> host(nd);
        std::memcpy(host.data(), rows.data(), (size_t)n * sizeof(DerivTRow));
        std::memcpy(host.data() + 3 * (size_t)n, bt.data(), bt.size() * sizeof(double));
        EMIX_CUDA_TRY(cudaMemcpy(buf, host.data(), nd * sizeof(double), cudaMemcpyHostToDevice));
        t.rows = reinterpret_cast<const DerivTRow *>(buf);
        t.bt = buf + 3 * (size_t)n;
        // the run of rows around the middle equal to the middle row, when
        // that row is the antisymmetric 5-point stencil
        const double *mid = bt.data() + 7 * (size_t)(n / 2);
        t.jlo = 1;
        t.jhi = 0;
        if (mid[0] == 0.0 && mid[3] == 0.0 && mid[6] == 0.0 && mid[4] == -mid[2] && mid[5] == -mid[1]) {
            auto same = [&](int j) { return std::memcmp(bt.data() + 7 * (size_t)j, mid, 7 * sizeof(double)) == 0; };
            int lo = n / 2, hi = n / 2;
            while (lo > 0 && same(lo - 1)) --lo;
            while (hi < n - 1 && same(hi + 1)) ++hi;
            t.jlo = lo;
            t.jhi = hi;
            t.ta = mid[2];
            t.tb = mid[1];
        }
    }
    std::lock_guard<std::mutex> lock(g_t_mu);
    g_t_tables[key] = t;
    *out = t;
    return EMIX_OK;
}

} // namespace emix
