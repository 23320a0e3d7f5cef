// Host-side set-up of libcrtomo_gb300: grid validation, band pattern with the
// ordered element contributions, the wavenumber rule and the Cuthill-McKee
// renumbering.  None of this is on the per-iteration path; it runs once per
// grid.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "crgpu_internal.h"

namespace crgpu {

// ---------------------------------------------------------------------------
// grid
// ---------------------------------------------------------------------------
int build_grid(const crgpu_grid *g, HostGrid &hg, std::string &msg) {
    if (!g || g->sanz <= 0 || g->typanz <= 0 || !g->typ || !g->nelanz || !g->selanz || !g->snr ||
        !g->sx || !g->sy || !g->nrel) {
        msg = "crgpu_grid: missing arrays";
        return ERR_ARG;
    }
    hg = HostGrid();
    hg.n = g->sanz;
    hg.mb = g->mb;
    int elanz = 0, relanz = 0, maxnk = 0;
    for (int i = 0; i < g->typanz; i++) {
        if (g->typ[i] > 10) relanz += g->nelanz[i];
        else elanz += g->nelanz[i];
        maxnk = std::max(maxnk, (int)g->selanz[i]);
    }
    if (g->ld_nrel < elanz + relanz || maxnk > 4) {
        msg = "crgpu_grid: ld_nrel < elanz+relanz or more than 4 nodes per element";
        return ERR_ARG;
    }
    hg.elanz = elanz;
    hg.relanz = relanz;
    hg.x.resize(hg.n);
    hg.y.resize(hg.n);
    for (int i = 0; i < hg.n; i++) {
        int s = g->snr[i];
        if (s < 1 || s > hg.n) {
            msg = "snr out of range";
            return ERR_ARG;
        }
        hg.x[i] = g->sx[s - 1];
        hg.y[i] = g->sy[s - 1];
    }
    hg.etype.resize(elanz);
    hg.enodes.assign((size_t)elanz * 4, -1);
    hg.btype.resize(relanz);
    hg.bnodes.assign((size_t)relanz * 2, -1);
    hg.brnr.assign(relanz, -1);
    hg.dirichlet.assign(hg.n, 0);
    int iel = 0, ie = 0, ib = 0;
    for (int t = 0; t < g->typanz; t++) {
        int ntyp = g->typ[t], nk = g->selanz[t];
        for (int j = 0; j < g->nelanz[t]; j++, iel++) {
            int nodes[4] = {-1, -1, -1, -1};
            for (int q = 0; q < nk; q++) {
                int nd = g->nrel[(size_t)q * g->ld_nrel + iel];
                if (nd < 1 || nd > hg.n) {
                    msg = "element node out of range";
                    return ERR_ARG;
                }
                nodes[q] = nd - 1;
            }
            if (ntyp <= 10) {
                if (ib > 0) {  // src/precal.f90:105-110 (rel <= 0)
                    msg = "boundary elements must follow the area elements";
                    return 36;
                }
                if (!((ntyp == 3 && nk == 3) || (ntyp == 5 && nk == 4) || (ntyp == 8 && nk == 4))) {
                    msg = "element type";  // src/precal.f90:190-193
                    return 18;
                }
                hg.etype[ie] = ntyp;
                for (int q = 0; q < 4; q++) hg.enodes[(size_t)ie * 4 + q] = nodes[q];
                ie++;
            } else {
                if (nk != 2 || (ntyp != 11 && ntyp != 12 && ntyp != 13)) {
                    msg = "boundary element type";
                    return 18;
                }
                hg.btype[ib] = ntyp;
                hg.bnodes[(size_t)ib * 2] = nodes[0];
                hg.bnodes[(size_t)ib * 2 + 1] = nodes[1];
                if (ntyp == 11) {
                    if (!g->rnr) {
                        msg = "rnr missing";
                        return ERR_ARG;
                    }
                    int r = g->rnr[ib];
                    if (r < 1 || r > elanz) {
                        msg = "border to element context is wrong";
                        return 111;
                    }
                    hg.brnr[ib] = r - 1;
                    hg.lbeta = true;
                    hg.nmixed++;
                }
                if (ntyp == 13) {
                    hg.lrandb = true;
                    hg.dirichlet[nodes[0]] = 1;
                    hg.dirichlet[nodes[1]] = 1;
                }
                ib++;
            }
        }
    }
    if (hg.lbeta && hg.lrandb) {  // src/precal.f90:90-95, 122-127
        msg = "mixed and Dirichlet boundaries together";
        return 101;
    }
    return 0;
}

// src/bsytop.f90:7-71: running mean of the type-12 element mid-heights
double host_sytop(const crgpu_grid *g) {
    double sytop = 0.0;
    int iel = 0;
    for (int t = 0; t < g->typanz; t++) {
        if (g->typ[t] == 12) {
            int nk = g->selanz[t];
            sytop = 0.0;
            for (int j = 1; j <= g->nelanz[t]; j++, iel++) {
                double sp = 0.0;
                for (int q = 0; q < nk; q++) {
                    int nd = g->nrel[(size_t)q * g->ld_nrel + iel];
                    sp += g->sy[g->snr[nd - 1] - 1];
                }
                sp = sp / nk;
                sytop = (j == 1) ? sp : (sytop * (j - 1) + sp) / j;
            }
        } else {
            iel += g->nelanz[t];
        }
    }
    return sytop;
}

// ---------------------------------------------------------------------------
// band pattern and element contributions (src/kompab.f90:80-138)
// ---------------------------------------------------------------------------
int build_pattern(const HostGrid &hg, Pattern &pat, std::string &msg) {
    const int n = hg.n, mb = hg.mb;
    struct Ent {
        int col;
        std::vector<int32_t> dom, bnd;
    };
    std::vector<std::vector<Ent>> rows(n);
    auto entry = [&](int r, int c) -> Ent & {
        for (auto &e : rows[r])
            if (e.col == c) return e;
        rows[r].push_back(Ent{c, {}, {}});
        return rows[r].back();
    };
    for (int i = 0; i < n; i++) entry(i, i);  // every diagonal exists
    for (int e = 0; e < hg.elanz; e++) {
        int nk = hg.etype[e] == 3 ? 3 : 4, imn = 0;
        for (int a = 0; a < nk; a++)
            for (int b = 0; b <= a; b++, imn++) {
                int p = hg.enodes[(size_t)e * 4 + a], q = hg.enodes[(size_t)e * 4 + b];
                if (std::abs(p - q) > mb) {
                    msg = "kompab: band width exceeded (element " + std::to_string(e + 1) + ")";
                    return 19;
                }
                entry(std::max(p, q), std::min(p, q)).dom.push_back((e << 4) | imn);
            }
    }
    for (int rb = 0; rb < hg.relanz; rb++) {
        if (hg.btype[rb] != 11) continue;  // src/kompab.f90:85 (types 12, 13 skipped)
        int imn = 0;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b <= a; b++, imn++) {
                int p = hg.bnodes[(size_t)rb * 2 + a], q = hg.bnodes[(size_t)rb * 2 + b];
                if (std::abs(p - q) > mb) {
                    msg = "kompab: band width exceeded (boundary element)";
                    return 19;
                }
                entry(std::max(p, q), std::min(p, q)).bnd.push_back((rb << 4) | imn);
            }
    }
    pat = Pattern();
    pat.n = n;
    // rows padded to a fixed width RW (padding entries have col = -1 and no
    // contributions) so that row i starts at i*RW without an indirection
    int rw = 1;
    for (int i = 0; i < n; i++) {
        std::sort(rows[i].begin(), rows[i].end(), [](const Ent &a, const Ent &b) { return a.col < b.col; });
        rw = std::max(rw, (int)rows[i].size());
    }
    if (rw > 31) {
        msg = "more than 31 lower-pattern entries in one row";
        return ERR_UNSUPPORTED;
    }
    pat.rw = rw;
    pat.rowptr.assign(n + 1, 0);
    for (int i = 0; i < n; i++) pat.rowptr[i + 1] = pat.rowptr[i] + rw;
    pat.nnz = pat.rowptr[n];
    pat.col.assign(pat.nnz, -1);
    pat.row.resize(pat.nnz);
    pat.dom_ptr.assign(pat.nnz + 1, 0);
    pat.bnd_ptr.assign(pat.nnz + 1, 0);
    int p = 0;
    for (int i = 0; i < n; i++)
        for (int q = 0; q < rw; q++, p++) {
            pat.row[p] = i;
            int nd = 0, nb = 0;
            if (q < (int)rows[i].size()) {
                const Ent &e = rows[i][q];
                pat.col[p] = e.col;
                nd = (int)e.dom.size();
                nb = (int)e.bnd.size();
                pat.dom_list.insert(pat.dom_list.end(), e.dom.begin(), e.dom.end());
                pat.bnd_list.insert(pat.bnd_list.end(), e.bnd.begin(), e.bnd.end());
            }
            pat.dom_ptr[p + 1] = pat.dom_ptr[p] + nd;
            pat.bnd_ptr[p + 1] = pat.bnd_ptr[p] + nb;
        }
    if (pat.dom_list.empty()) pat.dom_list.push_back(0);
    if (pat.bnd_list.empty()) pat.bnd_list.push_back(0);
    // full symmetric CSR
    std::vector<int> cnt(n, 0);
    for (int q = 0; q < pat.nnz; q++) {
        if (pat.col[q] < 0) continue;
        cnt[pat.row[q]]++;
        if (pat.col[q] != pat.row[q]) cnt[pat.col[q]]++;
    }
    pat.fptr.assign(n + 1, 0);
    for (int i = 0; i < n; i++) pat.fptr[i + 1] = pat.fptr[i] + cnt[i];
    pat.nnz_full = pat.fptr[n];
    pat.fcol.resize(pat.nnz_full);
    pat.fidx.resize(pat.nnz_full);
    std::vector<int> fill(pat.fptr.begin(), pat.fptr.end() - 1);
    for (int q = 0; q < pat.nnz; q++) {
        int r = pat.row[q], c = pat.col[q];
        if (c < 0) continue;
        pat.fcol[fill[r]] = c;
        pat.fidx[fill[r]++] = q;
        if (r != c) {
            pat.fcol[fill[c]] = r;
            pat.fidx[fill[c]++] = q;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Gauss rules by Golub-Welsch (symmetric tridiagonal Jacobi matrix, implicit
// QL), nodes polished by Newton on the three-term recurrence.
// ---------------------------------------------------------------------------
static void tql_eigen(int n, std::vector<double> &d, std::vector<double> &e, std::vector<double> &z0) {
    // d: diagonal, e: sub-diagonal (e[0..n-2]); z0: first components of the
    // eigenvectors (starts as e_1).
    e.push_back(0.0);
    for (int l = 0; l < n; l++) {
        for (int iter = 0; iter < 200; iter++) {
            int m = l;
            for (; m < n - 1; m++) {
                double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= 1e-17 * dd) break;
            }
            if (m == l) break;
            double gg = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::hypot(gg, 1.0);
            gg = d[m] - d[l] + e[l] / (gg + (gg >= 0 ? std::fabs(r) : -std::fabs(r)));
            double s = 1.0, c = 1.0, pp = 0.0;
            int i;
            for (i = m - 1; i >= l; i--) {
                double f = s * e[i], b = c * e[i];
                r = std::hypot(f, gg);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= pp;
                    e[m] = 0.0;
                    break;
                }
                s = f / r;
                c = gg / r;
                gg = d[i + 1] - pp;
                r = (d[i] - gg) * s + 2.0 * c * b;
                pp = s * r;
                d[i + 1] = gg + pp;
                gg = c * r - b;
                double zf = z0[i + 1];
                z0[i + 1] = s * z0[i] + c * zf;
                z0[i] = c * z0[i] - s * zf;
            }
            if (r == 0.0 && i >= l) continue;
            d[l] -= pp;
            e[l] = gg;
            e[m] = 0.0;
        }
    }
}

static void legendre_rule(int n, std::vector<double> &x, std::vector<double> &w) {
    std::vector<double> d(n, 0.0), e(n > 1 ? n - 1 : 0), z(n, 0.0);
    for (int k = 1; k < n; k++) e[k - 1] = k / std::sqrt(4.0 * k * k - 1.0);
    z[0] = 1.0;
    tql_eigen(n, d, e, z);
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; i++) {
        double t = d[idx[i]], dp = 1.0;
        for (int it = 0; it < 3; it++) {  // Newton polish on P_n
            double p0 = 1.0, p1 = t;
            for (int j = 2; j <= n; j++) {
                double p2 = ((2.0 * j - 1.0) * t * p1 - (j - 1.0) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (t * p1 - p0) / (t * t - 1.0);
            t -= p1 / dp;
        }
        double p0 = 1.0, p1 = t;
        for (int j = 2; j <= n; j++) {
            double p2 = ((2.0 * j - 1.0) * t * p1 - (j - 1.0) * p0) / j;
            p0 = p1;
            p1 = p2;
        }
        dp = n * (t * p1 - p0) / (t * t - 1.0);
        x[i] = t;
        w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
    }
}

static void laguerre_rule(int n, std::vector<double> &x, std::vector<double> &w) {
    std::vector<double> d(n), e(n > 1 ? n - 1 : 0), z(n, 0.0);
    for (int k = 0; k < n; k++) d[k] = 2.0 * k + 1.0;
    for (int k = 1; k < n; k++) e[k - 1] = (double)k;
    z[0] = 1.0;
    tql_eigen(n, d, e, z);
    std::sort(d.begin(), d.end());
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; i++) {
        double t = d[i], dl = 1.0;
        for (int it = 0; it < 4; it++) {
            double p0 = 1.0, p1 = 1.0 - t;
            for (int j = 2; j <= n; j++) {
                double p2 = ((2.0 * j - 1.0 - t) * p1 - (j - 1.0) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            dl = n * (p1 - p0) / t;
            t -= p1 / dl;
        }
        double p0 = 1.0, p1 = 1.0 - t;
        for (int j = 2; j <= n; j++) {
            double p2 = ((2.0 * j - 1.0 - t) * p1 - (j - 1.0) * p0) / j;
            p0 = p1;
            p1 = p2;
        }
        dl = n * (p1 - p0) / t;
        x[i] = t;
        w[i] = 1.0 / (t * dl * dl);
    }
}

// src/rwaven.f90:22-171
int host_rwaven(const HostGrid &hg, int eanz, const int32_t *enr, int nanz, const int32_t *strnr,
                const int32_t *vnr, double *kwn, double *kwnwi, int32_t *kwnanz) {
    double amin = 1e9, amax = 0.0;
    double xe[4] = {0, 0, 0, 0}, ye[4] = {0, 0, 0, 0};
    for (int i = 0; i < nanz; i++) {
        int el[4];
        el[0] = strnr[i] % 10000;
        el[1] = (strnr[i] - el[0]) / 10000;
        el[2] = vnr[i] % 10000;
        el[3] = (vnr[i] - el[2]) / 10000;
        for (int j = 0; j < 4; j++) {
            if (el[j] > eanz) return 46;
            if (el[j] > 0) {
                int nd = enr[el[j] - 1] - 1;
                xe[j] = hg.x[nd];
                ye[j] = hg.y[nd];
            }
        }
        for (int r = 2; r < 4; r++) {
            if (el[r] <= 0) continue;
            for (int j = 0; j < 2; j++) {
                if (el[j] <= 0) continue;
                double dx = xe[r] - xe[j], dy = ye[r] - ye[j];
                double dd = std::sqrt(dx * dx + dy * dy);
                amin = std::min(dd, amin);
                amax = std::max(dd, amax);
            }
        }
    }
    if (amin < 1e-12 || amax < 1e-12) return 73;
    const int lanz = 4;
    // int(real(6d0*dlog10(amax/amin))): single-precision conversion, truncation
    int ganz = (int)(float)(6.0 * std::log10(amax / amin));
    ganz = std::max(ganz, 2);
    ganz = std::min(ganz, 30 - lanz);
    double k0 = 1.0 / (2.0 * amin);
    std::vector<double> x, w;
    legendre_rule(ganz, x, w);  // on (-1, 1)
    for (int i = 0; i < ganz; i++) {
        double xi = 0.5 + 0.5 * x[i], wi = 0.5 * w[i];  // map to (0, 1)
        kwnwi[i] = 2.0 * k0 * wi * xi;
        kwn[i] = k0 * xi * xi;
    }
    laguerre_rule(lanz, x, w);
    for (int i = 0; i < lanz; i++) {
        kwnwi[ganz + i] = k0 * w[i] * std::exp(x[i]);
        kwn[ganz + i] = k0 * (x[i] + 1.0);
    }
    *kwnanz = ganz + lanz;
    return 0;
}

// ---------------------------------------------------------------------------
// Cuthill-McKee renumbering (cutmckee/cutmck.f:125-337)
//
// The graph keeps each node's neighbours in first-seen order with at most
// 500 slots; the start candidates are the first nodes of minimum degree
// (raising the degree until 100 candidates are found or it exceeds
// elanz/10), of which the last found is dropped; every sweep appends, for
// each node of the current level in order, its unnumbered neighbours by
// increasing degree with ties going to the LAST such neighbour in slot
// order; the first start with the smallest band width wins.
// ---------------------------------------------------------------------------
int host_cutmck(int32_t sanz, int32_t typanz, const int32_t *typ, const int32_t *nelanz,
                const int32_t *selanz, int32_t *nrel, int32_t ld_nrel, int32_t *snr, int32_t eanz,
                int32_t *enr, int32_t *mb_out) {
    constexpr int kSlots = 500, kStarts = 100;
    if (sanz <= 0) return ERR_ARG;
    int elanz = 0;
    for (int t = 0; t < typanz; t++)
        if (typ[t] <= 10) elanz += nelanz[t];
    std::vector<int32_t> adj((size_t)sanz * kSlots, 0);
    std::vector<int32_t> deg(sanz, 0);
    auto slot = [&](int node, int k) -> int32_t & { return adj[(size_t)node * kSlots + k]; };
    int base = 0;
    for (int t = 0; t < typanz; t++) {
        for (int e = 0; e < nelanz[t]; e++) {
            for (int a = 0; a < selanz[t] - 1; a++) {
                int u = nrel[(size_t)a * ld_nrel + base + e];
                for (int b = a + 1; b < selanz[t]; b++) {
                    int v = nrel[(size_t)b * ld_nrel + base + e];
                    bool known = false;
                    for (int k = 0; k < kSlots; k++) {
                        int32_t s = slot(u - 1, k);
                        if (s == v) {
                            known = true;
                            break;
                        }
                        if (s > 0) continue;
                        slot(u - 1, k) = v;
                        deg[u - 1]++;
                        break;
                    }
                    if (known) continue;
                    deg[v - 1]++;
                    if (deg[v - 1] <= kSlots) slot(v - 1, deg[v - 1] - 1) = u;
                }
            }
        }
        base += nelanz[t];
    }
    int dmin = *std::min_element(deg.begin(), deg.end());
    int dmax = *std::max_element(deg.begin(), deg.end());
    if (dmin == 0 || dmax > kSlots) return 5;
    std::vector<int> starts;
    for (;;) {
        bool full = false;
        for (int i = 0; i < sanz && !full; i++)
            if (deg[i] == dmin) {
                starts.push_back(i + 1);
                full = (int)starts.size() >= kStarts;
            }
        if (full || dmin > elanz / 10) break;
        dmin++;
    }
    int nstarts = (int)starts.size() - 1;
    if (nstarts < 1) return 5;
    std::vector<int32_t> order(sanz + 1), pos(sanz), best(sanz);
    std::vector<uint8_t> done(sanz);
    int best_mb = sanz;
    for (int is = 0; is < nstarts; is++) {
        std::fill(done.begin(), done.end(), 0);
        int s0 = starts[is];
        int cnt = 1;
        order[1] = s0;
        pos[s0 - 1] = 1;
        done[s0 - 1] = 1;
        int lev_begin = 1, lev_end = 1;
        while (lev_end < sanz) {
            for (int j = lev_begin; j <= lev_end; j++) {
                int u = order[j];
                for (;;) {
                    int bestd = kSlots, pick = 0;
                    for (int k = 0; k < deg[u - 1]; k++) {
                        int v = slot(u - 1, k);
                        if (done[v - 1] || deg[v - 1] > bestd) continue;
                        bestd = deg[v - 1];
                        pick = v;
                    }
                    if (!pick) break;
                    order[++cnt] = pick;
                    pos[pick - 1] = cnt;
                    done[pick - 1] = 1;
                }
            }
            int next_size = cnt - lev_end;
            if (next_size == 0) return 5;  // disconnected grid
            lev_begin = lev_end + 1;
            lev_end = lev_end + next_size;
        }
        int bw = 0;
        for (int i = 0; i < sanz; i++)
            for (int k = 0; k < deg[i]; k++) bw = std::max(bw, std::abs(pos[slot(i, k) - 1] - pos[i]));
        if (bw < best_mb) {
            best_mb = bw;
            best = pos;
        }
    }
    base = 0;
    for (int t = 0; t < typanz; t++) {
        for (int e = 0; e < nelanz[t]; e++)
            for (int q = 0; q < selanz[t]; q++) {
                int32_t &v = nrel[(size_t)q * ld_nrel + base + e];
                v = best[v - 1];
            }
        base += nelanz[t];
    }
    std::vector<int32_t> old(snr, snr + sanz);
    for (int i = 0; i < sanz; i++) snr[best[i] - 1] = old[i];
    for (int i = 0; i < eanz; i++) enr[i] = best[enr[i] - 1];
    *mb_out = best_mb;
    return 0;
}

// A second node order for the complex64 factor of wide bands: the nodes
// sorted by the coordinate along the mesh's longer extent, then by the other
// one.  On structured meshes this numbers the nodes line by line across the
// short side, a band of about one line instead of the two lines of a
// Cuthill-McKee level structure grown from a single node.  old_of_new[j] is
// the grid's node in position j; returns the band width of that order.
int host_geometric_order(const HostGrid &hg, std::vector<int32_t> &old_of_new, std::vector<int32_t> &new_of_old) {
    const int n = hg.n;
    double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
    for (int i = 0; i < n; i++) {
        x0 = std::min(x0, hg.x[i]);
        x1 = std::max(x1, hg.x[i]);
        y0 = std::min(y0, hg.y[i]);
        y1 = std::max(y1, hg.y[i]);
    }
    const bool along_x = (x1 - x0) >= (y1 - y0);
    old_of_new.resize(n);
    for (int i = 0; i < n; i++) old_of_new[i] = i;
    std::stable_sort(old_of_new.begin(), old_of_new.end(), [&](int a, int b) {
        const double pa = along_x ? hg.x[a] : hg.y[a], pb = along_x ? hg.x[b] : hg.y[b];
        if (pa != pb) return pa < pb;
        const double qa = along_x ? hg.y[a] : hg.x[a], qb = along_x ? hg.y[b] : hg.x[b];
        return qa < qb;
    });
    new_of_old.assign(n, 0);
    for (int j = 0; j < n; j++) new_of_old[old_of_new[j]] = j;
    int mb = 0;
    for (int e = 0; e < hg.elanz; e++) {
        int lo = n, hi = -1;
        for (int q = 0; q < 4; q++) {
            const int v = hg.enodes[(size_t)e * 4 + q];
            if (v < 0) continue;
            lo = std::min(lo, new_of_old[v]);
            hi = std::max(hi, new_of_old[v]);
        }
        mb = std::max(mb, hi - lo);
    }
    for (int b = 0; b < hg.relanz; b++) {
        const int u = hg.bnodes[(size_t)b * 2], v = hg.bnodes[(size_t)b * 2 + 1];
        if (u >= 0 && v >= 0) mb = std::max(mb, std::abs(new_of_old[u] - new_of_old[v]));
    }
    return mb;
}

// hg renumbered by new_of_old (coordinates, element and boundary nodes,
// Dirichlet flags), with band width mb
void host_permute_grid(HostGrid &hg, const std::vector<int32_t> &old_of_new, const std::vector<int32_t> &new_of_old,
                       int mb) {
    const int n = hg.n;
    std::vector<double> x(n), y(n);
    std::vector<uint8_t> dir(n);
    for (int j = 0; j < n; j++) {
        x[j] = hg.x[old_of_new[j]];
        y[j] = hg.y[old_of_new[j]];
        dir[j] = hg.dirichlet[old_of_new[j]];
    }
    hg.x.swap(x);
    hg.y.swap(y);
    hg.dirichlet.swap(dir);
    for (auto &v : hg.enodes)
        if (v >= 0) v = new_of_old[v];
    for (auto &v : hg.bnodes)
        if (v >= 0) v = new_of_old[v];
    hg.mb = mb;
}

}  // namespace crgpu
