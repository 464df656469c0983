// Network compiler: reaction-pair factor lists -> the gather tables the
// rate/source and Jacobian kernels read.
//
// Replaces the code generation of the reference (make_chem_funs.py:113-430,
// which writes chemdf/df as Python source, and :653-717, which differentiates
// df symbolically with sympy).  Instead of generated code we build, once per
// network:
//   * src   : for every species s the list of (pair p, +-coefficient), one
//             entry per written term, in the order the generated chemdf sums
//             them (reaction order; reactants before products, :288-305);
//   * w     : one derivative term d v_p / d y_q per (pair, distinct species);
//   * J     : for every structurally non-zero entry (s, q) of the per-layer
//             chemistry Jacobian the list of (w, stoichiometry) to gather.
// All tables are gathers, so the device kernels are deterministic (no atomics).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "vk_internal.cuh"

static thread_local std::string g_net_err;

// The tables in the form the rate kernel gathers them, so that every gathered
// term costs one FP64 instruction and the lanes of a warp run loops of equal
// length (FP64 issue is the rate kernel's bound on this chip):
//  * source term (pair p, coefficient e): acc = fma(c, v[slot], acc).  For a
//    power-of-two |e| the product e*v is exact, so the fma equals the generated
//    chemdf's "acc + e*v" bit for bit (slot p, c = e); any other |e| reads an
//    extra slot holding round(|e| v_p) with c = +-1, which is the same again.
//  * derivative half term: d v_p / d y_q from one side of the pair,
//    k_side x (product of the side's factors with q's exponent lowered by one),
//    M a factor like the species; the exponent of q moves into the Jacobian
//    gather coefficient (an exact integer product).
//  * Jacobian entry (s, q): sum over half terms of coefficient x half term,
//    coefficient = +-(net stoichiometry of s) x (exponent of q), minus for
//    the reverse side.
static bool pow2(int e) { return e > 0 && (e & (e - 1)) == 0; }

static void build_gather_form(vk_network *n) {
    const int ni = n->ni, np = n->npair;
    n->porder.resize(np);
    for (int p = 0; p < np; ++p) n->porder[p] = p;
    std::stable_sort(n->porder.begin(), n->porder.end(), [&](int a, int b) {
        return n->pairs[a].nt[0] + n->pairs[a].nt[1] > n->pairs[b].nt[0] + n->pairs[b].nt[1];
    });
    std::map<std::pair<int, int>, int> xslot;          // (pair, |e|) -> extra slot
    for (size_t e = 0; e < n->src_nu.size(); ++e) {
        const int p = n->src[e].x, c = (int)n->src_nu[e], a = c < 0 ? -c : c;
        if (pow2(a)) {
            n->src_slot.push_back(p);
            n->src_c.push_back((double)c);
        } else {
            auto it = xslot.find({p, a});
            int m;
            if (it == xslot.end()) {
                m = (int)n->xmul_pair.size();
                xslot[{p, a}] = m;
                n->xmul_pair.push_back(p);
                n->xmul_fac.push_back((double)a);
            } else {
                m = it->second;
            }
            n->src_slot.push_back(np + m);
            n->src_c.push_back(c < 0 ? -1.0 : 1.0);
        }
    }
    // half terms of every derivative term w
    struct Half { int k; int mult; std::vector<int16_t> fac; int w; int sign; };
    std::vector<Half> halves;
    for (int wi = 0; wi < (int)n->w.size(); ++wi) {
        const WDesc &wd = n->w[wi];
        const PairDesc &pd = n->pairs[wd.pair];
        for (int side = 0; side < 2; ++side) {
            const int pos = side ? wd.rpos : wd.fpos;
            if (pos < 0) continue;
            const int nf = side ? pd.nr : pd.nf;
            const int16_t *sp = side ? pd.rsp : pd.fsp;
            const uint8_t *nu = side ? pd.rnu : pd.fnu;
            Half h;
            h.k = 2 * wd.pair + side;
            h.w = wi;
            h.sign = side ? -1 : 1;
            h.mult = nu[pos];
            for (int i = 0; i < nf; ++i) {
                const int cnt = (i == pos) ? nu[i] - 1 : nu[i];
                for (int r = 0; r < cnt; ++r) h.fac.push_back(sp[i]);
            }
            const int mp = side ? pd.rm : pd.fm;
            for (int r = 0; r < mp; ++r) h.fac.push_back((int16_t)ni);
            halves.push_back(h);
        }
    }
    std::vector<int> hidx(halves.size());
    for (size_t i = 0; i < halves.size(); ++i) hidx[i] = (int)i;
    std::stable_sort(hidx.begin(), hidx.end(), [&](int a, int b) {
        return halves[a].fac.size() > halves[b].fac.size();
    });
    std::vector<std::vector<int>> of_w(n->w.size());   // w -> its half terms (new indices)
    n->hptr.push_back(0);
    for (size_t r = 0; r < hidx.size(); ++r) {
        const Half &h = halves[hidx[r]];
        n->hk.push_back(h.k);
        n->hfac.insert(n->hfac.end(), h.fac.begin(), h.fac.end());
        n->hptr.push_back((int)n->hfac.size());
        of_w[h.w].push_back((int)r);
    }
    n->hjptr.push_back(0);
    for (size_t e = 0; e + 1 < n->jptr.size(); ++e) {
        for (int t = n->jptr[e]; t < n->jptr[e + 1]; ++t) {
            const int wi = n->jterm[t].x;
            const double nu_s = n->jterm_nu[t];
            for (int r : of_w[wi]) {
                const Half &h = halves[hidx[r]];
                n->hjterm.push_back(r);
                n->hjcoef.push_back(nu_s * h.sign * h.mult);
            }
        }
        n->hjptr.push_back((int)n->hjterm.size());
    }
}

extern "C" const char *vk_network_last_error(void) { return g_net_err.c_str(); }

extern "C" int vk_network_compile(const vk_network_desc *d, vk_network **out) {
    if (!d || !out) { g_net_err = "null argument"; return VK_EINVAL; }
    *out = nullptr;
    if (d->ni <= 0 || d->ni > VK_MAX_NI) {
        g_net_err = "ni must be in 1.." + std::to_string(VK_MAX_NI);
        return VK_EINVAL;
    }
    if (d->npair <= 0) { g_net_err = "npair must be positive"; return VK_EINVAL; }
    if (d->natom < 0 || d->natom > VK_MAX_NATOM) {
        g_net_err = "natom out of range"; return VK_EINVAL;
    }
    vk_network *n = new (std::nothrow) vk_network();
    if (!n) { g_net_err = "host allocation failed"; return VK_ENOMEM; }
    const int ni = d->ni, np = d->npair;
    n->ni = ni; n->npair = np; n->natom = d->natom;
    n->pairs.resize(np);
    std::vector<std::vector<std::pair<int, int>>> nu(np);   // merged net stoichiometry
    std::vector<std::vector<int2>> per_sp(ni);              // written-order source terms
    for (int p = 0; p < np; ++p) {
        PairDesc &pd = n->pairs[p];
        std::memset(&pd, 0, sizeof(pd));
        for (int i = 0; i < VK_MAXF; ++i) { pd.fsp[i] = -1; pd.rsp[i] = -1; }
        for (int side = 0; side < 2; ++side) {
            const int *ptr = side ? d->prod_ptr : d->reac_ptr;
            const int *sp = side ? d->prod_sp : d->reac_sp;
            const int *cf = side ? d->prod_nu : d->reac_nu;
            int t0 = ptr[p], t1 = ptr[p + 1];
            if (t1 < t0 || t1 - t0 > VK_MAXT) {
                g_net_err = "pair " + std::to_string(p) + ": more than 5 terms on one side";
                delete n; return VK_EINVAL;
            }
            pd.nt[side] = (uint8_t)(t1 - t0);
            std::vector<std::pair<int, int>> merged;   // (species, exponent) first-seen order
            int mpow = 0;
            for (int t = t0; t < t1; ++t) {
                int s = sp[t], e = cf[t];
                if (s < -1 || s >= ni || e < 1 || e > 15) {
                    g_net_err = "pair " + std::to_string(p) + ": bad term";
                    delete n; return VK_EINVAL;
                }
                pd.tsp[side][t - t0] = (int16_t)s;
                pd.tnu[side][t - t0] = (uint8_t)e;
                if (s < 0) { mpow += e; continue; }
                // generated chemdf: reactant terms subtract, product terms add
                per_sp[s].push_back(make_int2(p, side ? e : -e));
                bool found = false;
                for (auto &m : merged) if (m.first == s) { m.second += e; found = true; }
                if (!found) merged.push_back({s, e});
            }
            if ((int)merged.size() > VK_MAXF || mpow > 3) {
                g_net_err = "pair " + std::to_string(p) + ": too many distinct species or M";
                delete n; return VK_EINVAL;
            }
            for (size_t i = 0; i < merged.size(); ++i) {
                if (side) { pd.rsp[i] = (int16_t)merged[i].first; pd.rnu[i] = (uint8_t)merged[i].second; }
                else      { pd.fsp[i] = (int16_t)merged[i].first; pd.fnu[i] = (uint8_t)merged[i].second; }
            }
            if (side) { pd.nr = (uint8_t)merged.size(); pd.rm = (uint8_t)mpow; }
            else      { pd.nf = (uint8_t)merged.size(); pd.fm = (uint8_t)mpow; }
        }
        std::map<int, int> net;
        for (int i = 0; i < pd.nf; ++i) net[pd.fsp[i]] -= pd.fnu[i];
        for (int i = 0; i < pd.nr; ++i) net[pd.rsp[i]] += pd.rnu[i];
        for (auto &kv : net)
            if (kv.second != 0) nu[p].push_back(kv);
    }
    n->src_ptr.assign(ni + 1, 0);
    for (int s = 0; s < ni; ++s) {
        n->src_ptr[s + 1] = n->src_ptr[s] + (int)per_sp[s].size();
        n->src.insert(n->src.end(), per_sp[s].begin(), per_sp[s].end());
    }
    // derivative terms and Jacobian entries
    std::map<std::pair<int, int>, std::vector<int2>> jac;   // (s,q) -> terms
    for (int p = 0; p < np; ++p) {
        if (nu[p].empty()) continue;           // e.g. He -> He: no contribution
        const PairDesc &pd = n->pairs[p];
        std::vector<int> qs;
        for (int i = 0; i < pd.nf; ++i) qs.push_back(pd.fsp[i]);
        for (int i = 0; i < pd.nr; ++i)
            if (std::find(qs.begin(), qs.end(), pd.rsp[i]) == qs.end()) qs.push_back(pd.rsp[i]);
        for (int q : qs) {
            WDesc wd;
            wd.pair = p; wd.q = q; wd.fpos = -1; wd.rpos = -1;
            for (int i = 0; i < pd.nf; ++i) if (pd.fsp[i] == q) wd.fpos = i;
            for (int i = 0; i < pd.nr; ++i) if (pd.rsp[i] == q) wd.rpos = i;
            int wi = (int)n->w.size();
            n->w.push_back(wd);
            for (auto &kv : nu[p]) jac[{kv.first, q}].push_back(make_int2(wi, kv.second));
        }
    }
    n->jptr.push_back(0);
    for (auto &e : jac) {
        n->jrow.push_back(e.first.first);
        n->jcol.push_back(e.first.second);
        n->jpos.push_back(e.first.first * ni + e.first.second);
        n->jterm.insert(n->jterm.end(), e.second.begin(), e.second.end());
        n->jptr.push_back((int)n->jterm.size());
    }
    n->jrowptr.assign(ni + 1, 0);
    for (int r : n->jrow) n->jrowptr[r + 1]++;
    for (int r = 0; r < ni; ++r) n->jrowptr[r + 1] += n->jrowptr[r];
    n->jmap.assign((size_t)ni * ni, -1);
    for (size_t e = 0; e < n->jpos.size(); ++e) n->jmap[n->jpos[e]] = (int)e;
    // coefficient codes: +1 / -1 are applied as a signed add (exact, no
    // multiply); other coefficients multiply from the double table
    for (auto &t : n->src) {
        n->src_nu.push_back((double)t.y);
        t.y = (t.y == 1 || t.y == -1) ? t.y : 0;
    }
    for (auto &t : n->jterm) {
        n->jterm_nu.push_back((double)t.y);
        t.y = (t.y == 1 || t.y == -1) ? t.y : 0;
    }
    build_gather_form(n);
    n->compo.assign(d->compo, d->compo + (size_t)ni * d->natom);
    *out = n;
    return VK_OK;
}

extern "C" int vk_network_info(const vk_network *n, int *nnz, int *nw, int *nsrc) {
    if (!n) return VK_EINVAL;
    if (nnz) *nnz = (int)n->jpos.size();
    if (nw) *nw = (int)n->w.size();
    if (nsrc) *nsrc = (int)n->src.size();
    return VK_OK;
}

extern "C" int vk_network_jac_pattern(const vk_network *n, int *rows, int *cols) {
    if (!n || !rows || !cols) return VK_EINVAL;
    std::copy(n->jrow.begin(), n->jrow.end(), rows);
    std::copy(n->jcol.begin(), n->jcol.end(), cols);
    return VK_OK;
}

// Host evaluation of the gather form, term for term in the order and with the
// FP64 operations the rate kernel uses (k_rates, vk_kernels.cu): the pair
// rates in written order, the source gather as fma with the power-of-two
// coefficients and the extra product slots, the derivative half terms and the
// Jacobian gather.  A diagnostic, so the tables can be checked without a GPU.
static double side_value(double kk, const PairDesc &pd, int side, const double *y, double M) {
    double v = kk;
    for (int t = 0; t < pd.nt[side]; ++t) {
        const int s = pd.tsp[side][t];
        const double f = s < 0 ? M : y[s];
        double p = f;
        for (int i = 1; i < pd.tnu[side][t]; ++i) p = p * f;
        v = v * p;
    }
    return v;
}

extern "C" int vk_network_eval_host(const vk_network *n, const double *y, const double *k, double M,
                                    double *dydt, double *neg_jac) {
    if (!n || !y || !k) return VK_EINVAL;
    const int ni = n->ni, np = n->npair;
    std::vector<double> yl(y, y + ni);
    yl.push_back(M);                                   // factor index ni stands for M
    std::vector<double> v(np + n->xmul_pair.size());
    for (int p = 0; p < np; ++p)
        v[p] = side_value(k[2 * p], n->pairs[p], 0, yl.data(), M) -
               side_value(k[2 * p + 1], n->pairs[p], 1, yl.data(), M);
    for (size_t m = 0; m < n->xmul_pair.size(); ++m) v[np + m] = n->xmul_fac[m] * v[n->xmul_pair[m]];
    if (dydt) {
        for (int s = 0; s < ni; ++s) {
            double acc = 0.0;
            for (int e = n->src_ptr[s]; e < n->src_ptr[s + 1]; ++e)
                acc = std::fma(n->src_c[e], v[n->src_slot[e]], acc);
            dydt[s] = acc;
        }
    }
    if (neg_jac) {
        std::vector<double> h(n->hk.size());
        for (size_t i = 0; i < n->hk.size(); ++i) {
            double d = k[n->hk[i]];
            for (int t = n->hptr[i]; t < n->hptr[i + 1]; ++t) d = d * yl[n->hfac[t]];
            h[i] = d;
        }
        for (size_t e = 0; e + 1 < n->hjptr.size(); ++e) {
            double acc = 0.0;
            for (int t = n->hjptr[e]; t < n->hjptr[e + 1]; ++t) acc = std::fma(n->hjcoef[t], h[n->hjterm[t]], acc);
            neg_jac[e] = -acc;
        }
    }
    return VK_OK;
}

extern "C" void vk_network_free(vk_network *n) { delete n; }
