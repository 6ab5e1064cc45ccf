// rbg_plan.cpp -- ParamTot planner: walks the output index space with the
// reference's trigger chain and folds it into deduplicated GPU work.
//
// Reference behaviour reproduced (rBergLib/rBergomiMT.cpp:490-520 and the
// single-threaded twin RBergomi.cpp:184-209):
//   HTrigger      -> new Wtilde for H(i)                       (Volterra pass)
//   H|T trigger   -> WS = T(i)^H(i) Wtilde, dt = T(i)/N
//   H|T|eta       -> v from (xi, H(i), eta(i), current dt)
//   every index   -> Ivdt, IsvdW from v; BS with rho(i), K(i)
// Triggers compare with index i-1 within 1e-10 (ParamTot.h:38-42), so a value
// that moves by <= 1e-10 keeps the earlier state, exactly as the reference.
#include <cmath>
#include <map>
#include <tuple>

#include "rbg_internal.hpp"

namespace rbg {

namespace {
constexpr double kEps = 0.0000000001;

struct PT {
    const rbg_params& p;
    double H(long I) const { return p.H[I / p.op_size]; }
    double eta(long I) const { return p.eta[I / p.op_size]; }
    double rho(long I) const { return p.rho[I / p.op_size]; }
    double T(long I) const { return p.T[I % p.op_size]; }
    double K(long I) const { return p.K[I % p.op_size]; }
    bool trigH(long I) const { return I == 0 || std::fabs(H(I) - H(I - 1)) > kEps; }
    bool trigEta(long I) const { return I == 0 || std::fabs(eta(I) - eta(I - 1)) > kEps; }
    bool trigT(long I) const { return I == 0 || std::fabs(T(I) - T(I - 1)) > kEps; }
    bool trigRho(long I) const { return I == 0 || std::fabs(rho(I) - rho(I - 1)) > kEps; }
};

// getGamma, rBergLib/rBergomiMT.cpp:143-149
void gamma_table(double H, int N, double* G)
{
    double alpha = H - 0.5;
    G[0] = 0.0;
    for (int i = 1; i < N; ++i) G[i] = (std::pow(i + 1.0, alpha + 1.0) - std::pow(i, alpha + 1.0)) / (alpha + 1.0);
}
// One Volterra pass for H (rBergLib/rBergomiMT.cpp:83-109).
VolGroup make_vol(double H, int N)
{
    VolGroup v{};
    v.H = H;
    const double s2H = std::sqrt(2.0 * H);
    const double rhoH = s2H / (H + 0.5);
    v.a1 = rhoH / s2H;
    v.a2 = std::sqrt(1.0 - rhoH * rhoH) / s2H;
    v.c = std::sqrt(2.0 * H) * std::pow(1.0 / N, H);
    return v;
}

// A variance path: WS = c T_s^H_s X, dt = T_s / N, v from (H_v, eta).
VGroup make_vgroup(const Plan& plan, int vol, double Hs, double Ts, double Hv, double eta, int N)
{
    VGroup g{};
    g.vol = vol;
    g.Hs = Hs;
    g.Ts = Ts;
    g.Hv = Hv;
    g.eta = eta;
    g.dt = Ts / N;
    g.sdt = std::sqrt(g.dt);
    g.scale = plan.vols[vol].c * std::pow(Ts, Hs);
    g.xi = plan.xi;
    g.nsteps = N;
    return g;
}

// Groups the variance paths by Volterra pass (stable order); newidx maps
// creation order to the final index.
void order_vgroups(Plan& plan, const std::vector<VGroup>& vgs, std::vector<int>& newidx)
{
    std::vector<int> order;
    for (size_t v = 0; v < plan.vols.size(); ++v) {
        plan.vols[v].vg_begin = (int)order.size();
        for (size_t g = 0; g < vgs.size(); ++g)
            if (vgs[g].vol == (int)v) order.push_back((int)g);
        plan.vols[v].vg_end = (int)order.size();
    }
    newidx.assign(vgs.size(), 0);
    for (size_t k = 0; k < order.size(); ++k) {
        newidx[order[k]] = (int)k;
        plan.vgs.push_back(vgs[order[k]]);
    }
}

// Gamma per Volterra pass and the compensator per variance group.
void fill_tables(Plan& plan)
{
    const int N = plan.N;
    plan.gamma.assign((size_t)plan.vols.size() * N, 0.0);
    for (size_t v = 0; v < plan.vols.size(); ++v) gamma_table(plan.vols[v].H, N, plan.gamma.data() + v * N);
    plan.comp.assign((size_t)plan.vgs.size() * N, 0.0);
    for (size_t g = 0; g < plan.vgs.size(); ++g) {
        const VGroup& G = plan.vgs[g];
        double* c = plan.comp.data() + g * N;
        // updateV's compensator, evaluated as the reference writes it:
        // 0.5 * eta * eta * pow((i - 1 + comp_shift) * dt, 2 * H) with j = i - 1
        for (int j = 0; j + 1 < N; ++j)
            c[j] = 0.5 * G.eta * G.eta * std::pow((j + plan.comp_shift) * G.dt, 2 * G.Hv);
    }
}
}  // namespace

bool build_plan(const rbg_params& p, Plan& plan, std::string& err, bool plain_mc)
{
    if (p.par_size <= 0 || p.op_size <= 0) { err = "par_size and op_size must be positive"; return false; }
    if (!p.H || !p.eta || !p.rho || !p.T || !p.K) { err = "null parameter array"; return false; }
    if (p.N < 1) { err = "N must be >= 1"; return false; }
    if (p.M < 1) { err = "M must be >= 1"; return false; }
    const long out = (long)p.par_size * p.op_size;
    if (out > (1L << 24)) { err = "par_size * op_size too large"; return false; }
    for (int q = 0; q < p.par_size; ++q)
        if (!(p.H[q] > 0.0 && p.H[q] < 1.0)) { err = "H must lie in (0, 1)"; return false; }

    plan = Plan();
    plan.xi = p.xi;
    plan.N = p.N;
    PT pt{p};

    std::map<double, int> vol_of_H;
    std::map<std::tuple<int, double, double, double, double>, int> vg_of_key;
    std::vector<VGroup> vgs;
    std::vector<int> out_vg(out);
    std::vector<double> out_rho(out);

    int cur_vol = -1, cur_vg = -1;
    double Hs = 0, Ts = 0, rho_s = 0;
    for (long i = 0; i < out; ++i) {
        bool update = pt.trigH(i);
        if (update) {
            auto it = vol_of_H.find(pt.H(i));
            if (it == vol_of_H.end()) {
                it = vol_of_H.emplace(pt.H(i), (int)plan.vols.size()).first;
                plan.vols.push_back(make_vol(pt.H(i), p.N));
            }
            cur_vol = it->second;
        }
        update = update || pt.trigT(i);
        if (update) {
            Hs = pt.H(i);
            Ts = pt.T(i);
        }
        update = update || pt.trigEta(i);
        if (update) {
            auto key = std::make_tuple(cur_vol, Hs, Ts, pt.H(i), pt.eta(i));
            auto it = vg_of_key.find(key);
            if (it == vg_of_key.end()) {
                it = vg_of_key.emplace(key, (int)vgs.size()).first;
                vgs.push_back(make_vgroup(plan, cur_vol, Hs, Ts, pt.H(i), pt.eta(i), p.N));
            }
            cur_vg = it->second;
        }
        // plain MC only: S is recomputed when rho moves by more than 1e-10
        // (rBergLib/rBergomiMT.cpp:256-262); RT prices use rho(i) directly
        update = update || pt.trigRho(i);
        if (update) rho_s = pt.rho(i);
        out_vg[i] = cur_vg;
        out_rho[i] = plain_mc ? rho_s : pt.rho(i);
    }

    std::vector<int> newidx;
    order_vgroups(plan, vgs, newidx);
    plan.outs.resize(out);
    for (long i = 0; i < out; ++i) {
        plan.outs[i].vg = newidx[out_vg[i]];
        plan.outs[i].rho = out_rho[i];
        plan.outs[i].K = pt.K(i);
        plan.outs[i].T = pt.T(i);
    }

    fill_tables(plan);
    return true;
}

bool build_plan_unordered(const rbg_unordered& u, Plan& plan, std::string& err, const double* xi_per,
                          int comp_shift)
{
    if (u.size <= 0) { err = "size must be positive"; return false; }
    if (!u.H || !u.eta || !u.rho || !u.T || !u.K) { err = "null parameter array"; return false; }
    if (u.N < 1) { err = "N must be >= 1"; return false; }
    if (u.M < 1) { err = "M must be >= 1"; return false; }
    if (u.size > (1L << 24)) { err = "size too large"; return false; }
    for (long i = 0; i < u.size; ++i)
        if (!(u.H[i] > 0.0 && u.H[i] < 1.0)) { err = "H must lie in (0, 1)"; return false; }

    plan = Plan();
    plan.xi = xi_per ? xi_per[0] : u.xi;
    plan.N = u.N;
    plan.comp_shift = comp_shift;
    // updatePayoffUnordered (rBergomi/rBergomiMT.cpp:940-957) recomputes the
    // whole chain for every index: Volterra pass by H(i), WS = T(i)^H(i) Wtilde,
    // dt = T(i)/N, v from (H(i), eta(i)).  Equal tuples give equal states, so
    // passes are shared by exact H and variance groups by exact (H, T, eta).
    std::map<double, int> vol_of_H;
    std::map<std::tuple<double, double, double, double>, int> vg_of_key;
    std::vector<VGroup> vgs;
    std::vector<int> out_vg(u.size);
    for (long i = 0; i < u.size; ++i) {
        const double H = u.H[i], T = u.T[i], eta = u.eta[i];
        auto it = vol_of_H.find(H);
        if (it == vol_of_H.end()) {
            it = vol_of_H.emplace(H, (int)plan.vols.size()).first;
            plan.vols.push_back(make_vol(H, u.N));
        }
        const double xi = xi_per ? xi_per[i] : u.xi;
        auto key = std::make_tuple(H, T, eta, xi);
        auto jt = vg_of_key.find(key);
        if (jt == vg_of_key.end()) {
            jt = vg_of_key.emplace(key, (int)vgs.size()).first;
            vgs.push_back(make_vgroup(plan, it->second, H, T, H, eta, u.N));
            vgs.back().xi = xi;
        }
        out_vg[i] = jt->second;
    }
    std::vector<int> newidx;
    order_vgroups(plan, vgs, newidx);
    plan.outs.resize(u.size);
    for (long i = 0; i < u.size; ++i) {
        plan.outs[i].vg = newidx[out_vg[i]];
        plan.outs[i].rho = u.rho[i];
        plan.outs[i].K = u.K[i];
        plan.outs[i].T = u.T[i];
    }
    fill_tables(plan);
    return true;
}

}  // namespace rbg
