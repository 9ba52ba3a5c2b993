/*
 * assist_oracle.cpp -- CPU restatement of ASSIST's equations-of-motion path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for libassist_gb300's device path and
 * the timed CPU baseline.  Nothing in the product links or calls it.
 *
 * What it restates (file:line in the ASSIST v1.2.0 sources):
 *   - .440 ("ASCII-derived binary") loader      src/ascii_ephem.c:105-252
 *   - Chebyshev position/velocity/acceleration  src/ascii_ephem.c:27-65
 *   - planet evaluation incl. Earth/Moon split  src/ascii_ephem.c:275-384
 *   - DAF/SPK type-2 loader                      src/spk.c:267-402
 *   - asteroid (position-only) evaluation        src/spk.c:405-481
 *   - planets from an SPK file: comment constants and masses, target
 *     evaluation with T/S/U recurrences, Earth/Moon about the Earth-Moon
 *     barycentre                                 src/spk.c:49-110, 137-200,
 *                                                492-693, 695-800;
 *                                                src/assist.c:252-292
 *   - body dispatch incl. asteroid+Sun offset    src/forces.c:175-263
 *   - force dispatcher and term order            src/forces.c:49-173
 *   - direct gravity (+ variational)             src/forces.c:266-433
 *   - Earth J2/J3/J4 (+ variational)             src/forces.c:435-642
 *   - Sun J2 (+ variational)                     src/forces.c:644-772
 *   - Marsden non-gravitational (+ variational)  src/forces.c:774-1057
 *   - GR potential / simple / EIH (+ variational) src/forces.c:1059-1983
 * plus the IAS15 integrator that ASSIST runs under (REBOUND, not vendored),
 * written from Rein & Spiegel (2015, MNRAS 446, 1424): Gauss-Radau substeps,
 * predictor-corrector iteration, the global step-size control ASSIST selects
 * (adaptive_mode = 1, src/assist.c:446) and the step-to-step b prediction.
 *
 * Everything is templated on the scalar type: double (the oracle), dd
 * (double-double, for error statements) and an operation-counting type (the
 * algorithmic flop counts quoted for the roofline).  Accumulation order per
 * particle follows the reference: non-grav, Earth harmonics, Sun J2, EIH, GR
 * potential, GR simple, then direct terms body by body (asteroids first, then
 * Pluto, Moon, Mars, Mercury, Neptune, Uranus, Earth, Venus, Saturn, Jupiter,
 * Sun).  Built with -ffp-contract=off so x86 and Arm give identical doubles.
 */
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "dd.h"

namespace {

enum { OK = 0, ERR_EPHEM_FILE = 1, ERR_AST_FILE = 2, ERR_NAST = 3, ERR_NEPHEM = 4, ERR_COVERAGE = 5 };
enum { B_SUN = 0, B_MER, B_VEN, B_EAR, B_MOO, B_MAR, B_JUP, B_SAT, B_URA, B_NEP, B_PLU, NPL = 11 };
enum { C_MER = 0, C_VEN, C_EMB, C_MAR, C_JUP, C_SAT, C_URA, C_NEP, C_PLU, C_LUN, C_SUN, C_NUT, C_LIB, C_MAN, C_TDB, NCOL };
enum { F_SUN = 0x01, F_PLANETS = 0x02, F_AST = 0x04, F_NONGRAV = 0x08, F_EARTH_H = 0x10, F_SUN_H = 0x20,
       F_EIH = 0x40, F_GR_SIMPLE = 0x80, F_GR_POT = 0x100 };

/* ---------------------------------------------------------------- counting */
struct OpTally { long long add, mul, div, sqrt, fn; };
static thread_local OpTally g_tally;
static thread_local OpTally g_tally_bodies;
static thread_local OpTally g_tally_shared;
struct cnt {
    double v;
    cnt() : v(0) {}
    cnt(double x) : v(x) {}
    explicit operator double() const { return v; }
};
static inline cnt operator+(cnt a, cnt b) { g_tally.add++; return cnt(a.v + b.v); }
static inline cnt operator-(cnt a, cnt b) { g_tally.add++; return cnt(a.v - b.v); }
static inline cnt operator-(cnt a) { return cnt(-a.v); }
static inline cnt operator*(cnt a, cnt b) { g_tally.mul++; return cnt(a.v * b.v); }
static inline cnt operator/(cnt a, cnt b) { g_tally.div++; return cnt(a.v / b.v); }
static inline cnt& operator+=(cnt& a, cnt b) { a = a + b; return a; }
static inline cnt& operator-=(cnt& a, cnt b) { a = a - b; return a; }
static inline cnt& operator*=(cnt& a, cnt b) { a = a * b; return a; }
static inline bool operator<(cnt a, cnt b) { return a.v < b.v; }
static inline bool operator>(cnt a, cnt b) { return a.v > b.v; }
static inline bool operator==(cnt a, cnt b) { return a.v == b.v; }
static inline bool operator!=(cnt a, cnt b) { return a.v != b.v; }
static inline cnt sqrt(cnt a) { g_tally.sqrt++; return cnt(std::sqrt(a.v)); }
static inline cnt pow(cnt a, double y) { g_tally.fn++; return cnt(std::pow(a.v, y)); }

/* Counting aid: move the operations tallied since `before` to the shared
 * tally, the work of a force evaluation that does not depend on the particle
 * (a kernel that shares one body table among many particles does it once per
 * table). */
static inline void tally_to_shared(const OpTally& before) {
    g_tally_shared.add += g_tally.add - before.add; g_tally_shared.mul += g_tally.mul - before.mul;
    g_tally_shared.div += g_tally.div - before.div; g_tally_shared.sqrt += g_tally.sqrt - before.sqrt;
    g_tally_shared.fn += g_tally.fn - before.fn;
    g_tally.add = before.add; g_tally.mul = before.mul; g_tally.div = before.div; g_tally.sqrt = before.sqrt;
    g_tally.fn = before.fn;
}
static inline cnt floor(cnt a) { return cnt(std::floor(a.v)); }
static inline double to_double(cnt a) { return a.v; }

using std::sqrt;
static inline double pow(double a, double y) { return std::pow(a, y); }

/* The origin-minus-body half (xo - x_body) of a particle-body separation:
 * the same subtraction, tallied when counting as particle-independent work. */
template <class T>
static inline T osub(const T& a, const T& b) {
    T r = a - b;
    if constexpr (std::is_same<T, cnt>::value) { g_tally.add--; g_tally_shared.add++; }
    return r;
}
static inline double floor(double a) { return std::floor(a); }

/* ---------------------------------------------------------------- files */
static bool read_all(const char* path, std::vector<unsigned char>& out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n <= 0) { std::fclose(f); return false; }
    out.resize((size_t)n);
    size_t got = std::fread(out.data(), 1, (size_t)n, f);
    std::fclose(f);
    return got == (size_t)n;
}
template <class X> static X rd(const std::vector<unsigned char>& b, size_t off) {
    X x; std::memcpy(&x, b.data() + off, sizeof(X)); return x;
}

/* .440 planets file: header fields as read by src/ascii_ephem.c:123-186 */
struct Ascii {
    double beg, end, inc, cau, cem;
    int num, ver;
    int off[NCOL], ncf[NCOL], niv[NCOL], ncm[NCOL];
    size_t rec;                            // record length in doubles
    std::vector<double> data;              // whole file as doubles (records 0..)
    std::vector<std::string> names;
    std::vector<double> con;
    double mass[NPL];
    double J2E, J3E, J4E, J2SUN, AU, RE, CLIGHT, ASUN;
    bool find(const char* name, double* out) const {
        char key[7] = "      ";
        for (int i = 0; i < 6 && name[i]; i++) key[i] = name[i];
        for (size_t p = 0; p < names.size(); p++)
            if (std::memcmp(names[p].data(), key, 6) == 0) { *out = con[p]; return true; }
        *out = 0.0; return false;
    }
};

static Ascii* ascii_load(const char* path) {
    std::vector<unsigned char> b;
    if (!read_all(path, b) || b.size() < 0xB28 + 24) return nullptr;
    Ascii* a = new Ascii();
    size_t o = 0x0A5C;
    a->beg = rd<double>(b, o); a->end = rd<double>(b, o + 8); a->inc = rd<double>(b, o + 16);
    a->num = rd<int32_t>(b, o + 24); a->cau = rd<double>(b, o + 28); a->cem = rd<double>(b, o + 36);
    o += 44;
    for (int p = 0; p < NCOL; p++) a->ncm[p] = 3;
    a->ncm[C_NUT] = 2; a->ncm[C_TDB] = 1;
    for (int p = 0; p < 12; p++, o += 12) {
        a->off[p] = rd<int32_t>(b, o); a->ncf[p] = rd<int32_t>(b, o + 4); a->niv[p] = rd<int32_t>(b, o + 8);
    }
    a->ver = rd<int32_t>(b, o); o += 4;
    a->off[12] = rd<int32_t>(b, o); a->ncf[12] = rd<int32_t>(b, o + 4); a->niv[12] = rd<int32_t>(b, o + 8);
    if (a->num < 0 || a->num > 100000) { delete a; return nullptr; }
    for (int p = 0; p < a->num; p++) {
        size_t no = p < 400 ? 0x00FC + 6 * (size_t)p : 0x0B28 + 6 * (size_t)(p - 400);
        a->names.emplace_back((const char*)b.data() + no, 6);
    }
    o = 0x0B28 + 6 * (size_t)(a->num > 400 ? a->num - 400 : 0);
    for (int p = 13; p < 15; p++, o += 12) {
        a->off[p] = rd<int32_t>(b, o); a->ncf[p] = rd<int32_t>(b, o + 4); a->niv[p] = rd<int32_t>(b, o + 8);
    }
    for (int p = 0; p < NCOL; p++) a->off[p] -= 1;
    size_t rec = 2;
    for (int p = 0; p < NCOL; p++) rec += (size_t)a->ncf[p] * a->niv[p] * a->ncm[p];
    a->rec = rec;
    a->data.resize(b.size() / 8);
    std::memcpy(a->data.data(), b.data(), a->data.size() * 8);
    for (int p = 0; p < a->num; p++) a->con.push_back(rd<double>(b, rec * 8 + 8 * (size_t)p));
    double v;
    a->find("GMS", &a->mass[B_SUN]); a->find("GM1", &a->mass[B_MER]); a->find("GM2", &a->mass[B_VEN]);
    double emrat, gmb;
    a->find("EMRAT", &emrat); a->find("GMB", &gmb);
    a->mass[B_EAR] = (emrat / (1. + emrat)) * gmb;
    a->mass[B_MOO] = 1. / (1 + emrat) * gmb;
    a->find("GM4", &a->mass[B_MAR]); a->find("GM5", &a->mass[B_JUP]); a->find("GM6", &a->mass[B_SAT]);
    a->find("GM7", &a->mass[B_URA]); a->find("GM8", &a->mass[B_NEP]); a->find("GM9", &a->mass[B_PLU]);
    a->find("J2E", &a->J2E); a->find("J3E", &a->J3E); a->find("J4E", &a->J4E); a->find("J2SUN", &a->J2SUN);
    a->find("AU", &a->AU); a->find("RE", &a->RE); a->find("CLIGHT", &a->CLIGHT); a->find("ASUN", &a->ASUN);
    (void)v;
    return a;
}

/* SPK type-2 file: summaries per target as collected by src/spk.c:295-376 */
struct SpkTarget { int code, cen; double mass, beg, end, res; std::vector<int> one, two; };
struct Spk { std::vector<SpkTarget> targets; std::vector<double> data; };

static Spk* spk_load(const char* path) {
    std::vector<unsigned char> b;
    if (!read_all(path, b) || b.size() < 1024) return nullptr;
    if (std::memcmp(b.data(), "DAF/SPK", 7) != 0) return nullptr;
    int nd = rd<int32_t>(b, 8), ni = rd<int32_t>(b, 12);
    if (8 * (nd + (ni + 1) / 2) != 40) return nullptr;
    int fward = rd<int32_t>(b, 76);
    Spk* s = new Spk();
    long recno = fward;
    while (recno > 0) {
        size_t ro = (size_t)(recno - 1) * 1024;
        if (ro + 1024 > b.size()) { delete s; return nullptr; }
        double next = rd<double>(b, ro), nsum = rd<double>(b, ro + 16);
        for (int k = 0; k < (int)nsum; k++) {
            size_t so = ro + 24 + 40 * (size_t)k;
            double sbeg = rd<double>(b, so), send = rd<double>(b, so + 8);
            int tar = rd<int32_t>(b, so + 16), cen = rd<int32_t>(b, so + 20);
            int one = rd<int32_t>(b, so + 32), two = rd<int32_t>(b, so + 36);
            SpkTarget* t = nullptr;
            for (auto& x : s->targets) if (x.code == tar) { t = &x; break; }
            if (!t) {
                SpkTarget nt;
                nt.code = tar; nt.cen = cen; nt.mass = 0; nt.end = 0;
                nt.beg = 2451545.0 + sbeg / 86400.0;
                nt.res = (2451545.0 + send / 86400.0) - nt.beg;
                s->targets.push_back(nt);
                t = &s->targets.back();
            }
            t->one.push_back(one); t->two.push_back(two);
            t->end = 2451545.0 + send / 86400.0;
        }
        recno = (long)next;
    }
    s->data.resize(b.size() / 8);
    std::memcpy(s->data.data(), b.data(), s->data.size() * 8);
    return s;
}

struct Ephem {
    double jd_ref = 2451545.0;
    Ascii* pl = nullptr;
    Spk* ast = nullptr;
    Spk* pls = nullptr;                 /* planets from an SPK file (else pl) */
    int tgt[NPL] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
    int emb = -1;
    double AU, EMRAT, J2E, J3E, J4E, J2SUN, RE, CLIGHT, ASUN, Re_eq, Rs_eq, c_AU_per_day, c_squared, over_c_squared;
    int n_ast() const { return ast ? (int)ast->targets.size() : 0; }
};

/* DAF comment area: records 2 .. fward-1, trailing NUL/EOT bytes of each
 * record dropped, NUL ends a line (src/spk.c:49-110). */
static std::string spk_comments(const std::vector<unsigned char>& b) {
    std::string out;
    if (b.size() < 1024) return out;
    const int fward = rd<int32_t>(b, 76);
    for (int r = 0; r < fward - 2; r++) {
        size_t o = (size_t)(1 + r) * 1024;
        if (o + 1024 > b.size()) break;
        int len = 1024;
        while (len > 0 && (b[o + len - 1] == 0 || b[o + len - 1] == 4)) len--;
        for (int k = 0; k < len; k++) out.push_back(b[o + k] == 0 ? '\n' : (char)b[o + k]);
    }
    return out;
}

/* "KEY value" lines after "Initial conditions and constants used for
 * integration:", D exponents read as E (src/spk.c:695-760). */
struct SpkConst { double AU = 0, EMRAT = 0, J2E = 0, J3E = 0, J4E = 0, J2SUN = 0, RE = 0, CLIGHT = 0, ASUN = 0;
                  std::vector<std::pair<std::string, double>> masses; };
static SpkConst spk_constants(const std::string& c) {
    SpkConst k;
    bool in = false;
    size_t pos = 0;
    while (pos < c.size()) {
        size_t e = c.find('\n', pos);
        if (e == std::string::npos) e = c.size();
        std::string line = c.substr(pos, e - pos);
        pos = e + 1;
        if (line.empty()) continue;
        if (line.find("Initial conditions and constants used for integration:") != std::string::npos) in = true;
        if (!in) continue;
        for (auto& ch : line) if (ch == 'D' || ch == 'd') ch = 'E';
        char key[64], val[64];
        if (std::sscanf(line.c_str(), "%63s %63s", key, val) != 2) continue;
        const double v = std::strtod(val, nullptr);
        std::string K(key);
        if (K == "cau" || K == "AU") k.AU = v;
        else if (K == "EMRAT") k.EMRAT = v;
        else if (K == "J2E") k.J2E = v;
        else if (K == "J3E") k.J3E = v;
        else if (K == "J4E") k.J4E = v;
        else if (K == "J2SUN") k.J2SUN = v;
        else if (K == "RE") k.RE = v;
        else if (K == "CLIGHT") k.CLIGHT = v;
        else if (K == "ASUN") k.ASUN = v;
        else if (K.compare(0, 2, "GM") == 0 || K.compare(0, 2, "MA") == 0) k.masses.push_back({K, v});
    }
    return k;
}

/* Masses of SPK targets from the parsed GMs (src/spk.c:137-200): planets by
 * name, Earth and Moon split from GMB by EMRAT, asteroids as MAnnnn. */
static void spk_join_masses(Spk* s, const SpkConst& k) {
    if (!s) return;
    static const struct { const char* name; int code; } pc[] = {
        {"GMS", 10}, {"GM1", 1}, {"GM2", 2}, {"GMB", 399}, {"GMB", 3}, {"GMB", 301}, {"GM4", 4},
        {"GM5", 5}, {"GM6", 6}, {"GM7", 7}, {"GM8", 8}, {"GM9", 9}};
    for (auto& t : s->targets) {
        if (t.mass != 0) continue;
        char label[64] = {0};
        for (auto& q : pc) if (t.code == q.code) { std::snprintf(label, sizeof(label), "%s", q.name); break; }
        if (!label[0]) std::snprintf(label, sizeof(label), "MA%04d", t.code - 2000000);
        for (auto& m : k.masses) {
            if (m.first != label) continue;
            if (t.code == 399) t.mass = m.second * (k.EMRAT / (1. + k.EMRAT));
            else if (t.code == 301) t.mass = m.second * (1. / (1. + k.EMRAT));
            else t.mass = m.second;
            break;
        }
    }
}

/* src/assist.c:252-292: planets from an SPK file. */
static Ephem* ephem_load_spk(const char* planets, const char* asteroids) {
    std::vector<unsigned char> b;
    if (!read_all(planets, b)) return nullptr;
    Spk* ps = spk_load(planets);
    if (!ps) return nullptr;
    Ephem* e = new Ephem();
    e->pls = ps;
    static const int naif[NPL] = {10, 1, 2, 399, 301, 4, 5, 6, 7, 8, 9};
    for (int k = 0; k < NPL; k++)
        for (int i = 0; i < (int)ps->targets.size(); i++)
            if (ps->targets[(size_t)i].code == naif[k]) { e->tgt[k] = i; break; }
    for (int i = 0; i < (int)ps->targets.size(); i++)
        if (ps->targets[(size_t)i].code == 3) { e->emb = i; break; }
    e->ast = asteroids ? spk_load(asteroids) : nullptr;
    const SpkConst k = spk_constants(spk_comments(b));
    e->AU = k.AU; e->EMRAT = k.EMRAT; e->J2E = k.J2E; e->J3E = k.J3E; e->J4E = k.J4E; e->J2SUN = k.J2SUN;
    e->RE = k.RE; e->CLIGHT = k.CLIGHT; e->ASUN = k.ASUN;
    e->Re_eq = e->RE / e->AU;
    e->Rs_eq = e->ASUN / e->AU;
    e->c_AU_per_day = (e->CLIGHT / e->AU) * 86400;
    e->c_squared = e->c_AU_per_day * e->c_AU_per_day;
    e->over_c_squared = 1.0 / e->c_squared;
    spk_join_masses(e->pls, k);
    spk_join_masses(e->ast, k);
    return e;
}

/* src/assist.c:252-348 for the .440 branch (and the SPK branch above). */
static Ephem* ephem_load(const char* planets, const char* asteroids) {
    {
        std::vector<unsigned char> b;
        if (read_all(planets, b) && b.size() >= 8 && std::memcmp(b.data(), "DAF/SPK", 7) == 0)
            return ephem_load_spk(planets, asteroids);
    }
    Ascii* a = ascii_load(planets);
    if (!a) return nullptr;
    Ephem* e = new Ephem();
    e->pl = a;
    e->ast = asteroids ? spk_load(asteroids) : nullptr;
    e->J2E = a->J2E; e->J3E = a->J3E; e->J4E = a->J4E; e->J2SUN = a->J2SUN; e->AU = a->AU; e->RE = a->RE;
    e->CLIGHT = a->CLIGHT; e->ASUN = a->ASUN; e->EMRAT = a->cem;
    e->Re_eq = e->RE / e->AU;
    e->Rs_eq = e->ASUN / e->AU;
    e->c_AU_per_day = (e->CLIGHT / e->AU) * 86400.0;
    e->c_squared = e->c_AU_per_day * e->c_AU_per_day;
    e->over_c_squared = 1.0 / e->c_squared;
    if (e->ast) {
        for (auto& t : e->ast->targets) {
            if (t.code >= 2000000) {
                char key[16];
                std::snprintf(key, sizeof(key), "MA%04d", t.code - 2000000);
                double gm;
                if (a->find(key, &gm)) t.mass = gm;
            }
        }
    }
    return e;
}

/* ---------------------------------------------------------------- bodies */

/* Sub-interval and normalised time of tt = record fraction x niv, as
 * src/ascii_ephem.c:35-39 forms them: tau = 2 fmod(tt, 1) - 1 (fmod(tt, 1) is
 * tt - trunc(tt), exactly) and b = (int)tt.  A time a rounding below a record
 * boundary can give a tiny negative tt: b = 0 and tau just below -1, the start
 * of the record.  At tt == niv exactly the reference reads one sub-interval
 * past the column; here b stays in the last sub-interval, at its end
 * (tau = +1). */
template <class T>
static T subinterval_tau(T tt, int niv, int* b) {
    *b = (int)to_double(tt);
    T ip = T(std::trunc(to_double(tt)));
    if (*b >= niv) { *b = niv - 1; ip = T((double)(niv - 1)); }
    return 2.0 * (tt - ip) - 1.0;
}

/* Chebyshev series for one column over its sub-interval: position (T),
 * velocity (S = dT/dtau, times c) and acceleration (U = d2T/dtau2, times c^2),
 * src/ascii_ephem.c:27-65. */
template <class T>
static void cheb_column(const double* P, int ncm, int ncf, int niv, T tfrac, double inc, T* u, T* v, T* w) {
    T Tp[32], Sp[32], Up[32];
    T tt = tfrac * (double)niv;
    int blk;
    T tau = subinterval_tau(tt, niv, &blk);
    double c = (double)(niv * 2) / inc / 86400.0;
    Tp[0] = 1.0; Tp[1] = tau;
    Sp[0] = 0.0; Sp[1] = 1.0;
    Up[0] = 0.0; Up[1] = 0.0; Up[2] = 4.0;
    for (int p = 2; p < ncf; p++) {
        Tp[p] = 2.0 * tau * Tp[p - 1] - Tp[p - 2];
        Sp[p] = 2.0 * tau * Sp[p - 1] + 2.0 * Tp[p - 1] - Sp[p - 2];
    }
    for (int p = 3; p < ncf; p++) Up[p] = 2.0 * tau * Up[p - 1] + 4.0 * Sp[p - 1] - Up[p - 2];
    for (int m = 0; m < ncm; m++) {
        T su = 0.0, sv = 0.0, sw = 0.0;
        const double* cf = P + ncf * (m + blk * ncm);
        for (int p = 0; p < ncf; p++) {
            su += Tp[p] * cf[p];
            sv += Sp[p] * cf[p] * c;
            sw += Up[p] * cf[p] * c * c;
        }
        u[m] = su; v[m] = sv; w[m] = sw;
    }
}

/* Planet state from the .440 records, src/ascii_ephem.c:275-384.
 * out: GM, x,y,z, vx,vy,vz, ax,ay,az (AU, day). */
template <class T>
static int ascii_body(const Ephem& e, T t, int body, T* out) {
    const Ascii& a = *e.pl;
    if (body < 0 || body >= NPL) return ERR_NEPHEM;
    out[0] = a.mass[body];
    double jd = to_double(T(e.jd_ref) + t);
    if (jd < a.beg || jd > a.end) return ERR_COVERAGE;
    uint32_t blk = (uint32_t)to_double((T(e.jd_ref) + t - a.beg) / a.inc);
    size_t nrec = a.data.size() / a.rec;
    if ((size_t)blk + 2 >= nrec) return ERR_COVERAGE;       // past the last stored record
    const double* z = a.data.data() + (size_t)(blk + 2) * a.rec;
    T tf = ((T(e.jd_ref) - a.beg - (double)blk * a.inc) + t) / a.inc;
    static const int col_of[NPL] = {C_SUN, C_MER, C_VEN, -1, -1, C_MAR, C_JUP, C_SAT, C_URA, C_NEP, C_PLU};
    T u[3], v[3], w[3];
    if (body == B_EAR || body == B_MOO) {
        T eu[3], ev[3], ew[3], lu[3], lv[3], lw[3];
        cheb_column(z + a.off[C_EMB], 3, a.ncf[C_EMB], a.niv[C_EMB], tf, a.inc, eu, ev, ew);
        cheb_column(z + a.off[C_LUN], 3, a.ncf[C_LUN], a.niv[C_LUN], tf, a.inc, lu, lv, lw);
        double f = body == B_EAR ? -1.0 / (1.0 + a.cem) : a.cem / (1.0 + a.cem);
        for (int k = 0; k < 3; k++) { u[k] = eu[k] + lu[k] * f; v[k] = ev[k] + lv[k] * f; w[k] = ew[k] + lw[k] * f; }
    } else {
        int c = col_of[body];
        cheb_column(z + a.off[c], 3, a.ncf[c], a.niv[c], tf, a.inc, u, v, w);
    }
    for (int k = 0; k < 3; k++) {
        out[1 + k] = u[k] / a.cau;
        out[4 + k] = v[k] / (a.cau / 86400.);
        out[7 + k] = w[k] / (a.cau / (86400. * 86400.));
    }
    return OK;
}

/* As ascii_body, evaluating velocity and acceleration only when asked (the
 * position sums are the same operations either way). */
template <class T>
static void cheb_column_need(const double* P, int ncm, int ncf, int niv, T tfrac, double inc, T* u, T* v, T* w,
                             bool vel) {
    if (vel) { cheb_column(P, ncm, ncf, niv, tfrac, inc, u, v, w); return; }
    T Tp[32];
    T tt = tfrac * (double)niv;
    int blk;
    T tau = subinterval_tau(tt, niv, &blk);
    Tp[0] = 1.0; Tp[1] = tau;
    for (int p = 2; p < ncf; p++) Tp[p] = 2.0 * tau * Tp[p - 1] - Tp[p - 2];
    for (int m = 0; m < ncm; m++) {
        T su = 0.0;
        const double* cf = P + ncf * (m + blk * ncm);
        for (int p = 0; p < ncf; p++) su += Tp[p] * cf[p];
        u[m] = su;
    }
}

template <class T>
static int ascii_body_need(const Ephem& e, T t, int body, T* out, bool vel, bool acc) {
    if (acc) return ascii_body(e, t, body, out);
    const Ascii& a = *e.pl;
    if (body < 0 || body >= NPL) return ERR_NEPHEM;
    out[0] = a.mass[body];
    double jd = to_double(T(e.jd_ref) + t);
    if (jd < a.beg || jd > a.end) return ERR_COVERAGE;
    uint32_t blk = (uint32_t)to_double((T(e.jd_ref) + t - a.beg) / a.inc);
    size_t nrec = a.data.size() / a.rec;
    if ((size_t)blk + 2 >= nrec) return ERR_COVERAGE;
    const double* z = a.data.data() + (size_t)(blk + 2) * a.rec;
    T tf = ((T(e.jd_ref) - a.beg - (double)blk * a.inc) + t) / a.inc;
    static const int col_of[NPL] = {C_SUN, C_MER, C_VEN, -1, -1, C_MAR, C_JUP, C_SAT, C_URA, C_NEP, C_PLU};
    T u[3], v[3], w[3];
    if (body == B_EAR || body == B_MOO) {
        T eu[3], ev[3], ew[3], lu[3], lv[3], lw[3];
        cheb_column_need(z + a.off[C_EMB], 3, a.ncf[C_EMB], a.niv[C_EMB], tf, a.inc, eu, ev, ew, vel);
        cheb_column_need(z + a.off[C_LUN], 3, a.ncf[C_LUN], a.niv[C_LUN], tf, a.inc, lu, lv, lw, vel);
        double f = body == B_EAR ? -1.0 / (1.0 + a.cem) : a.cem / (1.0 + a.cem);
        for (int k = 0; k < 3; k++) {
            u[k] = eu[k] + lu[k] * f;
            if (vel) { v[k] = ev[k] + lv[k] * f; w[k] = ew[k] + lw[k] * f; }
        }
    } else {
        int c = col_of[body];
        cheb_column_need(z + a.off[c], 3, a.ncf[c], a.niv[c], tf, a.inc, u, v, w, vel);
    }
    for (int k = 0; k < 3; k++) {
        out[1 + k] = u[k] / a.cau;
        if (vel) {
            out[4 + k] = v[k] / (a.cau / 86400.);
            out[7 + k] = w[k] / (a.cau / (86400. * 86400.));
        } else {
            out[4 + k] = NAN; out[7 + k] = NAN;
        }
    }
    return OK;
}

/* Asteroid heliocentric position, src/spk.c:405-481 (AU fixed at 149597870.7 km). */
template <class T>
static int spk_position(const Ephem& e, T t, int m, T* gm, T* pos) {
    const Spk* s = e.ast;
    if (!s) return ERR_AST_FILE;
    if (m < 0 || m >= (int)s->targets.size()) return ERR_NAST;
    const SpkTarget& tg = s->targets[m];
    double jd = to_double(T(e.jd_ref) + t);
    if (jd < tg.beg || jd > tg.end) return ERR_COVERAGE;
    *gm = tg.mass;
    int n = (int)to_double((T(e.jd_ref) + t - tg.beg) / tg.res);
    if (n >= (int)tg.two.size()) n = (int)tg.two.size() - 1;
    const double* dir = s->data.data() + tg.two[n] - 1;
    int R = (int)dir[-1];
    int P = (R - 2) / 3;
    double init_jd = 2451545.0 + dir[-3] / 86400.0;
    int nrec = (int)dir[0];
    int b = (int)to_double(((T(e.jd_ref) - init_jd) + t) / (dir[-2] / 86400.0));
    if (b >= nrec) b = nrec - 1;
    const double* val = s->data.data() + (tg.one[n] - 1) + (size_t)b * R;
    T z = ((T(e.jd_ref) - (2451545.0 + val[0] / 86400.0)) + t) / (val[1] / 86400.0);
    T Tp[32];
    Tp[0] = 1.0; Tp[1] = z;
    for (int p = 2; p < P; p++) Tp[p] = 2.0 * z * Tp[p - 1] - Tp[p - 2];
    for (int k = 0; k < 3; k++) {
        T acc = 0.0;
        for (int p = 0; p < P; p++) acc += Tp[p] * val[2 + k * P + p];
        pos[k] = acc / 149597870.7;
    }
    return OK;
}

/* Position, velocity, acceleration sums of one SPK target (km, km/s,
 * km/s^2) with the T, S, U recurrences of src/spk.c:492-548. */
template <class T>
static void spk_target_pos(const Spk& s, const SpkTarget& tg, const Ephem& e, T t, T* u, T* v, T* w) {
    int n = (int)to_double((T(e.jd_ref) + t - tg.beg) / tg.res);
    if (n >= (int)tg.two.size()) n = (int)tg.two.size() - 1;    // at the very end (the reference reads past)
    const double* dir = s.data.data() + tg.two[n] - 1;
    const int R = (int)dir[-1];
    const int P = (R - 2) / 3;
    int b = (int)to_double(((T(e.jd_ref) - (2451545.0 + dir[-3] / 86400.0)) + t) / (dir[-2] / 86400.0));
    const int nrec = (int)dir[0];
    if (b >= nrec) b = nrec - 1;
    const double* val = s.data.data() + (tg.one[n] - 1) + (size_t)b * R;
    T z = ((T(e.jd_ref) - (2451545.0 + val[0] / 86400.0)) + t) / (val[1] / 86400.0);
    const double c = 1.0 / val[1];
    T Tp[32], Sp[32], Up[32];
    Tp[0] = 1.0; Tp[1] = z;
    Sp[0] = 0.0; Sp[1] = 1.0;
    Up[0] = 0.0; Up[1] = 0.0; Up[2] = 4.0;
    for (int p = 2; p < P; p++) {
        Tp[p] = 2.0 * z * Tp[p - 1] - Tp[p - 2];
        Sp[p] = 2.0 * z * Sp[p - 1] + 2.0 * Tp[p - 1] - Sp[p - 2];
    }
    for (int p = 3; p < P; p++) Up[p] = 2.0 * z * Up[p - 1] + 4.0 * Sp[p - 1] - Up[p - 2];
    for (int k = 0; k < 3; k++) {
        const int b0 = 2 + k * P;
        T su = 0.0, sv = 0.0, sw = 0.0;
        for (int p = 0; p < P; p++) {
            const double coeff = val[b0 + p];
            su += coeff * Tp[p];
            sv += coeff * Sp[p] * c;
            sw += coeff * Up[p] * c * c;
        }
        u[k] = su; v[k] = sv; w[k] = sw;
    }
}

/* Planet state from an SPK planets file, src/spk.c:550-693: the target of
 * the ASSIST body (Earth 399 and Moon 301 plus the Earth-Moon barycentre),
 * in AU and days.  out: GM, x,y,z, vx,vy,vz, ax,ay,az. */
template <class T>
static int spk_body(const Ephem& e, T t, int body, T* out) {
    if (body < 0 || body >= NPL || e.tgt[body] < 0) return ERR_NEPHEM;
    const Spk& s = *e.pls;
    const SpkTarget& tg = s.targets[(size_t)e.tgt[body]];
    double jd = to_double(T(e.jd_ref) + t);
    if (jd < tg.beg || jd > tg.end) return ERR_COVERAGE;
    out[0] = tg.mass;
    T u[3], v[3], w[3];
    spk_target_pos(s, tg, e, t, u, v, w);
    if (body == B_EAR || body == B_MOO) {
        T eu[3], ev[3], ew[3];
        spk_target_pos(s, s.targets[(size_t)e.emb], e, t, eu, ev, ew);
        for (int k = 0; k < 3; k++) { u[k] += eu[k]; v[k] += ev[k]; w[k] += ew[k]; }
    }
    const double au = e.AU, spd = 86400.;
    for (int k = 0; k < 3; k++) {
        out[1 + k] = u[k] / au;
        out[4 + k] = v[k] / (au / spd);
        out[7 + k] = w[k] / (au / (spd * spd));
    }
    return OK;
}

/* Planet i from whichever planets file is loaded. */
template <class T>
static int planet_body(const Ephem& e, T t, int body, T* out) {
    return e.pls ? spk_body(e, t, body, out) : ascii_body(e, t, body, out);
}
template <class T>
static int planet_body_need(const Ephem& e, T t, int body, T* out, bool vel, bool acc) {
    return e.pls ? spk_body(e, t, body, out) : ascii_body_need(e, t, body, out, vel, acc);
}

/* Body i at time t, src/forces.c:175-263 (no cache: the reference's cache
 * returns bit-identical values, unit_tests/ephem_cache). */
template <class T>
static int body_state(const Ephem& e, int i, T t, T* out) {
    if (i < NPL) return planet_body(e, t, i, out);
    T gm, p[3];
    int f = spk_position(e, t, i - NPL, &gm, p);
    if (f != OK) return f;
    T sun[10];
    f = planet_body(e, t, B_SUN, sun);
    if (f != OK) return f;
    out[0] = gm;
    out[1] = p[0] + sun[1]; out[2] = p[1] + sun[2]; out[3] = p[2] + sun[3];
    for (int k = 4; k < 10; k++) out[k] = NAN;
    return OK;
}

/* ---------------------------------------------------------------- forces */
struct ForceOpts { int forces, gr_eih_sources, geocentric; double alpha, nk, nm, nn, r0; };

/* Does the force model read body i's velocity?  The Sun's (non-grav, GR
 * simple, EIH), the EIH sources' and, geocentric, the Earth's. */
static bool need_velocity(const ForceOpts& o, int i) {
    if (i == B_SUN) return true;
    if ((o.forces & F_EIH) && i < o.gr_eih_sources) return true;
    if (o.geocentric == 1 && i == B_EAR) return true;
    return false;
}

/* Accelerations of n_real real particles (x, v: 3*n_real) and n_var first
 * order variational particles (vx, vv: 3*n_var; var k belongs to real
 * particle vtp[k], particle_params row n_real + k) at time t; acc receives
 * 3*(n_real + n_var) values (zeroed first, as REBOUND does). */
template <class T>
static int forces(const Ephem& e, const ForceOpts& o, T t, int n_real, const T* x, const T* v,
                  int n_var, const int* vtp, const T* vx, const T* vv, const double* params, T* acc) {
    const int nb = NPL + e.n_ast();
    std::vector<T> B((size_t)nb * 10);
    /* Body states at t.  The reference evaluates position, velocity and
     * acceleration of every planet (src/ascii_ephem.c:27-65) and, for every
     * asteroid, the Sun again (src/forces.c:216); positions do not depend on
     * the velocity/acceleration sums, so evaluating each planet once, with
     * only the derivatives the force model reads, gives identical values and
     * an operation count without the reference's redundant work. */
    for (int i = 0; i < NPL; i++) {
        int f = planet_body_need(e, t, i, &B[(size_t)i * 10], need_velocity(o, i), o.geocentric == 1 && i == B_EAR);
        if (f != OK) return f;
    }
    for (int i = NPL; i < nb; i++) {
        T gm, p[3];
        int f = spk_position(e, t, i - NPL, &gm, p);
        if (f != OK) return f;
        T* out = &B[(size_t)i * 10];
        out[0] = gm;
        out[1] = p[0] + B[1]; out[2] = p[1] + B[2]; out[3] = p[2] + B[3];
        for (int k = 4; k < 10; k++) out[k] = NAN;
    }
    if constexpr (std::is_same<T, cnt>::value) g_tally_bodies = g_tally;   /* the body-state part of the count */
    auto GM = [&](int i) { return B[(size_t)i * 10]; };
    auto BX = [&](int i, int k) { return B[(size_t)i * 10 + 1 + k]; };
    auto BV = [&](int i, int k) { return B[(size_t)i * 10 + 4 + k]; };
    auto BA = [&](int i, int k) { return B[(size_t)i * 10 + 7 + k]; };
    const int ntot = n_real + n_var;
    for (int k = 0; k < 3 * ntot; k++) acc[k] = 0.0;
    T* avar = acc + 3 * n_real;
    // var particles grouped per real particle, in configuration order
    std::vector<std::vector<int>> vars((size_t)n_real);
    for (int k = 0; k < n_var; k++) if (vtp[k] >= 0 && vtp[k] < n_real) vars[(size_t)vtp[k]].push_back(k);

    T xo[3] = {0.0, 0.0, 0.0}, vo[3] = {0.0, 0.0, 0.0}, ao[3] = {0.0, 0.0, 0.0};
    if (o.geocentric == 1)
        for (int k = 0; k < 3; k++) { xo[k] = BX(B_EAR, k); vo[k] = BV(B_EAR, k); ao[k] = BA(B_EAR, k); }

    // ---- Marsden non-gravitational, src/forces.c:774-1057
    if ((o.forces & F_NONGRAV) && params) {
        for (int j = 0; j < n_real; j++) {
            double A1 = params[3 * j], A2 = params[3 * j + 1], A3 = params[3 * j + 2];
            if (A1 == 0. && A2 == 0. && A3 == 0.) continue;
            T dx = x[3 * j] + osub(xo[0], BX(B_SUN, 0));
            T dy = x[3 * j + 1] + osub(xo[1], BX(B_SUN, 1));
            T dz = x[3 * j + 2] + osub(xo[2], BX(B_SUN, 2));
            T r2 = dx * dx + dy * dy + dz * dz;
            T r = sqrt(r2);
            T rr0 = r / o.r0;
            T g = o.alpha * pow(rr0, -o.nm) * pow(1.0 + pow(rr0, o.nn), -o.nk);
            T dvx = v[3 * j] + osub(vo[0], BV(B_SUN, 0));
            T dvy = v[3 * j + 1] + osub(vo[1], BV(B_SUN, 1));
            T dvz = v[3 * j + 2] + osub(vo[2], BV(B_SUN, 2));
            T hx = dy * dvz - dz * dvy, hy = dz * dvx - dx * dvz, hz = dx * dvy - dy * dvx;
            T h = sqrt(hx * hx + hy * hy + hz * hz);
            T tx = hy * dz - hz * dy, ty = hz * dx - hx * dz, tz = hx * dy - hy * dx;
            T tn = sqrt(tx * tx + ty * ty + tz * tz);
            acc[3 * j] += A1 * g * dx / r + A2 * g * tx / tn + A3 * g * hx / h;
            acc[3 * j + 1] += A1 * g * dy / r + A2 * g * ty / tn + A3 * g * hy / h;
            acc[3 * j + 2] += A1 * g * dz / r + A2 * g * tz / tn + A3 * g * hz / h;
            if (vars[(size_t)j].empty()) continue;
            T r3 = r * r * r;
            T v2 = dvx * dvx + dvy * dvy + dvz * dvz;
            T rdv = dx * dvx + dy * dvy + dz * dvz;
            T vdt = dvx * tx + dvy * ty + dvz * tz;
            T dgdr = (o.alpha / o.r0) * (-o.nm * pow(rr0, -o.nm - 1) * pow(1.0 + pow(rr0, o.nn), -o.nk)
                      + pow(rr0, -o.nm) * (-o.nk * o.nn) * pow(rr0, o.nn - 1) * pow(1.0 + pow(rr0, o.nn), -o.nk - 1));
            T dg[3] = {dgdr * dx / r, dgdr * dy / r, dgdr * dz / r};
            T h3 = h * h * h, t3 = tn * tn * tn;
            T hh3[3] = {hx / h3, hy / h3, hz / h3};
            T tt3[3] = {tx / t3, ty / t3, tz / t3};
            T d[3] = {dx, dy, dz}, dv[3] = {dvx, dvy, dvz}, hv[3] = {hx, hy, hz}, tv[3] = {tx, ty, tz};
            // partials d(a_a)/d(x_b), d(a_a)/d(v_b), d(a_a)/dA_k
            T Jx[3][3], Jv[3][3], JA[3][3];
            for (int aa = 0; aa < 3; aa++) {
                JA[aa][0] = g * d[aa] / r; JA[aa][1] = g * tv[aa] / tn; JA[aa][2] = g * hv[aa] / h;
            }
            // diagonal position partials (src/forces.c:942-952)
            for (int aa = 0; aa < 3; aa++) {
                Jx[aa][aa] = A1 * (dg[aa] * d[aa] / r + g * (1. / r - d[aa] * d[aa] / r3))
                    + A2 * (dg[aa] * tv[aa] / tn + g * ((d[aa] * dv[aa] - rdv) / tn - tt3[aa] * (2. * d[aa] * vdt - rdv * tv[aa])))
                    + A3 * (dg[aa] * hv[aa] / h + g * (-hh3[aa]) * (v2 * d[aa] - rdv * dv[aa]));
            }
            // off-diagonal position partials (src/forces.c:954-976); eps(a,b) fixes the
            // sign of the cross-product term dv_c/h for the pair (a,b)
            static const int third[3][3] = {{-1, 2, 1}, {2, -1, 0}, {1, 0, -1}};
            static const double hsgn[3][3] = {{0, 1, -1}, {-1, 0, 1}, {1, -1, 0}};
            for (int aa = 0; aa < 3; aa++)
                for (int bb = 0; bb < 3; bb++) {
                    if (aa == bb) continue;
                    int cc = third[aa][bb];
                    Jx[aa][bb] = A1 * (dg[bb] * d[aa] / r + g * (-d[aa] * d[bb] / r3))
                        + A2 * (dg[bb] * tv[aa] / tn + g * ((2 * d[bb] * dv[aa] - d[aa] * dv[bb]) / tn - tt3[aa] * (2 * d[bb] * vdt - rdv * tv[bb])))
                        + A3 * (dg[bb] * hv[aa] / h + g * (hsgn[aa][bb] * dv[cc] / h - hh3[aa] * (v2 * d[bb] - rdv * dv[bb])));
                }
            // velocity partials (src/forces.c:978-1012)
            for (int aa = 0; aa < 3; aa++)
                for (int bb = 0; bb < 3; bb++) {
                    if (aa == bb) {
                        int p = (aa + 1) % 3, q = (aa + 2) % 3;
                        T ss = (aa == 0) ? d[1] * d[1] + d[2] * d[2] : (aa == 1) ? d[0] * d[0] + d[2] * d[2] : d[0] * d[0] + d[1] * d[1];
                        (void)p; (void)q;
                        Jv[aa][aa] = A1 * (0.) + A2 * g * (ss / tn - tt3[aa] * r2 * tv[aa])
                                     + A3 * g * (-hh3[aa] * (r2 * dv[aa] - d[aa] * rdv));
                    } else {
                        int cc = third[aa][bb];
                        Jv[aa][bb] = A1 * (0.) + A2 * g * (-d[bb] * d[aa] / tn - tt3[bb] * r2 * tv[aa])
                                     + A3 * g * (-hsgn[aa][bb] * d[cc] / h - hh3[aa] * (r2 * dv[bb] - d[bb] * rdv));
                    }
                }
            for (int k : vars[(size_t)j]) {
                double dA[3] = {params[3 * (n_real + k)], params[3 * (n_real + k) + 1], params[3 * (n_real + k) + 2]};
                for (int aa = 0; aa < 3; aa++) {
                    T s = vx[3 * k] * Jx[aa][0] + vx[3 * k + 1] * Jx[aa][1] + vx[3 * k + 2] * Jx[aa][2]
                        + vv[3 * k] * Jv[aa][0] + vv[3 * k + 1] * Jv[aa][1] + vv[3 * k + 2] * Jv[aa][2]
                        + dA[0] * JA[aa][0] + dA[1] * JA[aa][1] + dA[2] * JA[aa][2];
                    avar[3 * k + aa] += s;
                }
            }
        }
    }

    // ---- Earth J2/J3/J4 about the J2000 pole, src/forces.c:435-642
    if (o.forces & F_EARTH_H) {
        const T GMe = GM(B_EAR);
        const double J2 = e.J2E, J3 = e.J3E, J4 = e.J4E, Re = e.Re_eq;
        const double ra = 0.0 * M_PI / 180., dec = 90.0 * M_PI / 180.;
        const double ca = std::cos(ra), sa = std::sin(ra), cd = std::cos(dec), sd = std::sin(dec);
        for (int j = 0; j < n_real; j++) {
            T dx = x[3 * j] + osub(xo[0], BX(B_EAR, 0));
            T dy = x[3 * j + 1] + osub(xo[1], BX(B_EAR, 1));
            T dz = x[3 * j + 2] + osub(xo[2], BX(B_EAR, 2));
            T r2 = dx * dx + dy * dy + dz * dz;
            T r = sqrt(r2);
            T px = -dx * sa + dy * ca;
            T py = -dx * ca * sd - dy * sa * sd + dz * cd;
            T pz = dx * ca * cd + dy * sa * cd + dz * sd;
            T c2 = pz * pz / r2;
            T p2 = 3. * J2 * Re * Re / r2 / r2 / r / 2.;
            T f2 = 5. * c2 - 1.;
            T rx = GMe * p2 * f2 * px, ry = GMe * p2 * f2 * py, rz = GMe * p2 * (f2 - 2.) * pz;
            T p3 = 5. * J3 * Re * Re * Re / r2 / r2 / r / 2.;
            T f3 = 3. - 7. * c2;
            rx += -GMe * p3 * (1. / r2) * f3 * px * pz;
            ry += -GMe * p3 * (1. / r2) * f3 * py * pz;
            rz += -GMe * p3 * (6. * c2 - 7. * c2 * c2 - 0.6);
            T p4 = 5. * J4 * Re * Re * Re * Re / r2 / r2 / r2 / r / 8.;
            T f4 = 63. * c2 * c2 - 42. * c2 + 3.;
            rx += GMe * p4 * f4 * px;
            ry += GMe * p4 * f4 * py;
            rz += GMe * p4 * (f4 + 12. - 28. * c2) * pz;
            acc[3 * j] += -rx * sa - ry * ca * sd + rz * ca * cd;
            acc[3 * j + 1] += rx * ca - ry * sa * sd + rz * sa * cd;
            acc[3 * j + 2] += ry * cd + rz * sd;
            if (vars[(size_t)j].empty()) continue;
            T g2 = 7. * c2 - 1.;
            T g3 = 35. * c2 * c2 - 30. * c2 + 3.;
            T m2[3][3];
            m2[0][0] = GMe * p2 * (f2 - 5. * g2 * px * px / r2);
            m2[1][1] = GMe * p2 * (f2 - 5. * g2 * py * py / r2);
            m2[2][2] = GMe * p2 * (-1.) * g3;
            m2[0][1] = m2[1][0] = GMe * p2 * (-5.) * g2 * px * py / r2;
            m2[1][2] = m2[2][1] = GMe * p2 * (-5.) * (g2 - 2.) * py * pz / r2;
            m2[0][2] = m2[2][0] = GMe * p2 * (-5.) * (g2 - 2.) * px * pz / r2;
            T ct = pz / r;
            T h2 = 21 * (-3. * c2 + 1.) / r2;
            T h3 = 3 * (-21. * c2 * c2 + 14. * c2 - 1.) / r2;
            T h4 = (-63. * c2 * c2 + 70. * c2 - 15.) * ct / r;
            T m3[3][3];
            m3[0][0] = GMe * p3 * ct * (h2 * px * px - f3) / r;
            m3[1][1] = GMe * p3 * ct * (h2 * py * py - f3) / r;
            m3[2][2] = GMe * p3 * h4;
            m3[0][1] = m3[1][0] = GMe * p3 * h2 * ct * px * py / r;
            m3[1][2] = m3[2][1] = GMe * p3 * h3 * py;
            m3[0][2] = m3[2][0] = GMe * p3 * h3 * px;
            T k2 = 33. * c2 * c2 - 18. * c2 + 1.;
            T k3 = 33. * c2 * c2 - 30. * c2 + 5.;
            T k4 = 231. * c2 * c2 * c2 - 315. * c2 * c2 + 105. * c2 - 5.;
            T m4[3][3];
            m4[0][0] = GMe * p4 * (f4 - 21. * k2 * px * px / r2);
            m4[1][1] = GMe * p4 * (f4 - 21. * k2 * py * py / r2);
            m4[2][2] = GMe * p4 * (-3.) * k4;
            m4[0][1] = m4[1][0] = GMe * p4 * (-21.) * k2 * px * py / r2;
            m4[1][2] = m4[2][1] = GMe * p4 * (-21.) * k3 * py * pz / r2;
            m4[0][2] = m4[2][0] = GMe * p4 * (-21.) * k3 * px * pz / r2;
            for (int k : vars[(size_t)j]) {
                T ddx = vx[3 * k], ddy = vx[3 * k + 1], ddz = vx[3 * k + 2];
                T q[3] = {-ddx * sa + ddy * ca, -ddx * ca * sd - ddy * sa * sd + ddz * cd, ddx * ca * cd + ddy * sa * cd + ddz * sd};
                T da[3];
                for (int aa = 0; aa < 3; aa++) {
                    da[aa] = q[0] * m2[aa][0] + q[1] * m2[aa][1] + q[2] * m2[aa][2];
                    da[aa] += q[0] * m3[aa][0] + q[1] * m3[aa][1] + q[2] * m3[aa][2];
                    da[aa] += q[0] * m4[aa][0] + q[1] * m4[aa][1] + q[2] * m4[aa][2];
                }
                avar[3 * k] += -da[0] * sa - da[1] * ca * sd + da[2] * ca * cd;
                avar[3 * k + 1] += da[0] * ca - da[1] * sa * sd + da[2] * sa * cd;
                avar[3 * k + 2] += da[1] * cd + da[2] * sd;
            }
        }
    }

    // ---- Sun J2, src/forces.c:644-772
    if (o.forces & F_SUN_H) {
        const T GMs = GM(B_SUN);
        const double Rs = e.Rs_eq, J2 = e.J2SUN;
        const double ra = 286.13 * M_PI / 180., dec = 63.87 * M_PI / 180.;
        const double ca = std::cos(ra), sa = std::sin(ra), cd = std::cos(dec), sd = std::sin(dec);
        for (int j = 0; j < n_real; j++) {
            T dx = x[3 * j] + osub(xo[0], BX(B_SUN, 0));
            T dy = x[3 * j + 1] + osub(xo[1], BX(B_SUN, 1));
            T dz = x[3 * j + 2] + osub(xo[2], BX(B_SUN, 2));
            T r2 = dx * dx + dy * dy + dz * dz;
            T r = sqrt(r2);
            T px = -dx * sa + dy * ca;
            T py = -dx * ca * sd - dy * sa * sd + dz * cd;
            T pz = dx * ca * cd + dy * sa * cd + dz * sd;
            T c2 = pz * pz / r2;
            T p2 = 3. * J2 * Rs * Rs / r2 / r2 / r / 2.;
            T f2 = 5. * c2 - 1.;
            T g2 = 7. * c2 - 1.;
            T g3 = 35. * c2 * c2 - 30. * c2 + 3.;
            T rx = GMs * p2 * f2 * px, ry = GMs * p2 * f2 * py, rz = GMs * p2 * (f2 - 2.) * pz;
            acc[3 * j] += -rx * sa - ry * ca * sd + rz * ca * cd;
            acc[3 * j + 1] += rx * ca - ry * sa * sd + rz * sa * cd;
            acc[3 * j + 2] += ry * cd + rz * sd;
            if (vars[(size_t)j].empty()) continue;
            T m[3][3];
            m[0][0] = GMs * p2 * (f2 - 5. * g2 * px * px / r2);
            m[1][1] = GMs * p2 * (f2 - 5. * g2 * py * py / r2);
            m[2][2] = GMs * p2 * (-1.) * g3;
            m[0][1] = m[1][0] = GMs * p2 * (-5.) * g2 * px * py / r2;
            m[1][2] = m[2][1] = GMs * p2 * (-5.) * (g2 - 2.) * py * pz / r2;
            m[0][2] = m[2][0] = GMs * p2 * (-5.) * (g2 - 2.) * px * pz / r2;
            for (int k : vars[(size_t)j]) {
                T ddx = vx[3 * k], ddy = vx[3 * k + 1], ddz = vx[3 * k + 2];
                T q[3] = {-ddx * sa + ddy * ca, -ddx * ca * sd - ddy * sa * sd + ddz * cd, ddx * ca * cd + ddy * sa * cd + ddz * sd};
                T da[3];
                for (int aa = 0; aa < 3; aa++) da[aa] = q[0] * m[aa][0] + q[1] * m[aa][1] + q[2] * m[aa][2];
                avar[3 * k] += -da[0] * sa - da[1] * ca * sd + da[2] * ca * cd;
                avar[3 * k + 1] += da[0] * ca - da[1] * sa * sd + da[2] * sa * cd;
                avar[3 * k + 2] += da[1] * cd + da[2] * sd;
            }
        }
    }

    // ---- EIH / PPN (beta = gamma = 1), src/forces.c:1288-1983
    if (o.forces & F_EIH) {
        const double oc2 = e.over_c_squared;
        const double beta = 1.0, gamma = 1.0;
        for (int i = 0; i < n_real; i++) {
            const bool want_var = !vars[(size_t)i].empty();
            T t7[3] = {0.0, 0.0, 0.0}, t8[3] = {0.0, 0.0, 0.0};
            T J[3][6];
            T dt7[3][6], dt8[3][3];
            for (int a = 0; a < 3; a++) { for (int b = 0; b < 6; b++) { J[a][b] = 0.0; dt7[a][b] = 0.0; } for (int b = 0; b < 3; b++) dt8[a][b] = 0.0; }
            T vi[3] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
            for (int jj = 0; jj < o.gr_eih_sources; jj++) {
                T dij[3] = {x[3 * i] + osub(xo[0], BX(jj, 0)), x[3 * i + 1] + osub(xo[1], BX(jj, 1)), x[3 * i + 2] + osub(xo[2], BX(jj, 2))};
                T rij2 = dij[0] * dij[0] + dij[1] * dij[1] + dij[2] * dij[2];
                T rij = sqrt(rij2);
                T pre = GM(jj) / (rij2 * rij);
                T vj[3] = {BV(jj, 0) - vo[0], BV(jj, 1) - vo[1], BV(jj, 2) - vo[2]};
                T vi2 = vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2];
                T term2 = gamma * oc2 * vi2;
                T vj2 = vj[0] * vj[0] + vj[1] * vj[1] + vj[2] * vj[2];
                T term3 = (1 + gamma) * oc2 * vj2;
                T vivj = vi[0] * vj[0] + vi[1] * vj[1] + vi[2] * vj[2];
                T term4 = -2 * (1 + gamma) * oc2 * vivj;
                T rdvj = dij[0] * vj[0] + dij[1] * vj[1] + dij[2] * vj[2];
                T term5 = -1.5 * oc2 * (rdvj * rdvj) / (rij * rij);
                T fv[3];
                for (int a = 0; a < 3; a++) fv[a] = (2 + 2 * gamma) * vi[a] - (1 + 2 * gamma) * vj[a];
                T f = dij[0] * fv[0] + dij[1] * fv[1] + dij[2] * fv[2];
                T pf = pre * f;
                for (int a = 0; a < 3; a++) t7[a] += pf * (vi[a] - vj[a]);
                T term0 = 0.0, term1 = 0.0;
                T aj[3] = {0.0, 0.0, 0.0};
                T dterm0[3] = {0.0, 0.0, 0.0};
                for (int k = 0; k < NPL; k++) {
                    T dik[3] = {x[3 * i] + osub(xo[0], BX(k, 0)), x[3 * i + 1] + osub(xo[1], BX(k, 1)), x[3 * i + 2] + osub(xo[2], BX(k, 2))};
                    T rik2 = dik[0] * dik[0] + dik[1] * dik[1] + dik[2] * dik[2];
                    T rik = sqrt(rik2);
                    term0 += GM(k) / rik;
                    if (want_var) for (int a = 0; a < 3; a++) dterm0[a] -= GM(k) / (rik * rik * rik) * dik[a];
                    if (k != jj) {
                        /* source-source sums: the same for every particle */
                        OpTally before{};
                        if constexpr (std::is_same<T, cnt>::value) before = g_tally;
                        T djk[3] = {BX(jj, 0) - BX(k, 0), BX(jj, 1) - BX(k, 1), BX(jj, 2) - BX(k, 2)};
                        T rjk2 = djk[0] * djk[0] + djk[1] * djk[1] + djk[2] * djk[2];
                        T rjk = sqrt(rjk2);
                        term1 += GM(k) / rjk;
                        T fac = GM(k) / (rjk2 * rjk);
                        for (int a = 0; a < 3; a++) aj[a] -= fac * djk[a];
                        if constexpr (std::is_same<T, cnt>::value) tally_to_shared(before);
                    }
                }
                term0 *= -2 * (beta + gamma) * oc2;
                term1 *= -(2 * beta - 1) * oc2;
                T rdaj = dij[0] * (aj[0] - ao[0]) + dij[1] * (aj[1] - ao[1]) + dij[2] * (aj[2] - ao[2]);
                T term6 = -0.5 * oc2 * rdaj;
                T t8f = GM(jj) / rij * (3 + 4 * gamma) / 2;
                for (int a = 0; a < 3; a++) t8[a] += t8f * aj[a];
                T factor = term0 + term1 + term2 + term3 + term4 + term5 + term6;
                for (int a = 0; a < 3; a++) acc[3 * i + a] += -pre * dij[a] * factor;
                if (!want_var) continue;
                // variational partials of the source-j term (src/forces.c:1577-1913)
                T rij5 = rij * rij * rij * rij * rij;
                T dpre[3];
                for (int a = 0; a < 3; a++) dpre[a] = -3.0 * GM(jj) / rij5 * dij[a];
                for (int a = 0; a < 3; a++) dterm0[a] *= -2 * (beta + gamma) * oc2;
                T t5f = 3.0 * oc2 * rdvj / rij;
                T dfac[6];
                for (int a = 0; a < 3; a++) {
                    T dterm5 = -t5f * (vj[a] / rij - rdvj * dij[a] / (rij * rij * rij));
                    T dterm6 = -0.5 * oc2 * (aj[a] - ao[a]);
                    dfac[a] = dterm0[a] + T(0.0) + dterm5 + dterm6;
                    T dterm2 = 2.0 * gamma * oc2 * vi[a];
                    T dterm4 = -2 * (1 + gamma) * oc2 * vj[a];
                    dfac[3 + a] = T(0.0) + dterm2 + dterm4;
                }
                T pre3 = GM(jj) / (rij * rij * rij);   // as the variational pass forms it
                for (int a = 0; a < 3; a++) {
                    T rel = vi[a] - vj[a];
                    for (int b = 0; b < 3; b++) {
                        dt7[a][b] += dpre[b] * f * rel + pre3 * fv[b] * rel;
                        T dfdv = dij[b] * (2 + 2 * gamma);
                        dt7[a][3 + b] += pre3 * dfdv * rel + (a == b ? pre3 * f : T(0.0));
                        dt8[a][b] += -GM(jj) * aj[a] / (rij * rij * rij) * dij[b] * (3 + 4 * gamma) / 2;
                    }
                }
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 6; b++) {
                        T s;
                        if (b >= 3) s = -pre3 * dij[a] * dfac[b];
                        else if (b == a) s = -dpre[b] * dij[a] * factor - pre3 * factor - pre3 * dij[a] * dfac[b];
                        else s = -dpre[b] * dij[a] * factor - pre3 * dij[a] * dfac[b];
                        J[a][b] += s;
                    }
            }
            for (int a = 0; a < 3; a++) acc[3 * i + a] += t7[a] * oc2 + t8[a] * oc2;
            if (!want_var) continue;
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 6; b++) J[a][b] += b < 3 ? dt7[a][b] * oc2 + dt8[a][b] * oc2 : dt7[a][b] * oc2;
            for (int k : vars[(size_t)i])
                for (int a = 0; a < 3; a++)
                    avar[3 * k + a] += vx[3 * k] * J[a][0] + vx[3 * k + 1] * J[a][1] + vx[3 * k + 2] * J[a][2]
                                       + vv[3 * k] * J[a][3] + vv[3 * k + 1] * J[a][4] + vv[3 * k + 2] * J[a][5];
        }
    }

    // ---- GR potential (Nobili & Roxburgh), src/forces.c:1059-1161
    if (o.forces & F_GR_POT) {
        const double C2 = e.c_squared;
        const T GMs = GM(B_SUN);
        for (int j = 0; j < n_real; j++) {
            T p[3] = {x[3 * j] + osub(xo[0], BX(B_SUN, 0)), x[3 * j + 1] + osub(xo[1], BX(B_SUN, 1)), x[3 * j + 2] + osub(xo[2], BX(B_SUN, 2))};
            T r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
            T r = sqrt(r2);
            T pre = -6.0 * GMs * GMs / (C2 * r2 * r2);
            for (int a = 0; a < 3; a++) acc[3 * j + a] += pre * p[a];
            if (vars[(size_t)j].empty()) continue;
            T m[3][3];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    T s = -4.0 * pre * (p[a] / r) * (p[b] / r);
                    m[a][b] = a == b ? pre + s : s;
                }
            for (int k : vars[(size_t)j])
                for (int a = 0; a < 3; a++)
                    avar[3 * k + a] += vx[3 * k] * m[a][0] + vx[3 * k + 1] * m[a][1] + vx[3 * k + 2] * m[a][2];
        }
    }

    // ---- GR simple (Damour & Deruelle), src/forces.c:1163-1286
    if (o.forces & F_GR_SIMPLE) {
        const double C2 = e.c_squared;
        const T GMs = GM(B_SUN);
        for (int j = 0; j < n_real; j++) {
            T p[3], pv[3];
            for (int a = 0; a < 3; a++) {
                p[a] = x[3 * j + a] + osub(xo[a], BX(B_SUN, a));
                pv[a] = v[3 * j + a] + osub(vo[a], BV(B_SUN, a));
            }
            T v2 = pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2];
            T r = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
            T A = 4.0 * GMs / r - v2;
            T Bc = 4.0 * (p[0] * pv[0] + p[1] * pv[1] + p[2] * pv[2]);
            T pre = GMs / (r * r * r * C2);
            for (int a = 0; a < 3; a++) acc[3 * j + a] += pre * (A * p[a] + Bc * pv[a]);
            if (vars[(size_t)j].empty()) continue;
            T dpdr = -3.0 * pre / r;
            T m[3][6];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    T xr = p[a] * (p[b] / r) * 4.0 * GMs / (r * r);
                    T base = a == b ? (A - xr) + 4.0 * pv[b] * pv[a] : -xr + 4.0 * pv[b] * pv[a];
                    m[a][b] = dpdr * p[b] / r * (A * p[a] + Bc * pv[a]) + pre * base;
                    T vb = -2.0 * pv[b] * p[a] + 4.0 * p[b] * pv[a];
                    if (a == b) vb = vb + Bc;
                    m[a][3 + b] = pre * vb;
                }
            for (int k : vars[(size_t)j])
                for (int a = 0; a < 3; a++)
                    avar[3 * k + a] += vx[3 * k] * m[a][0] + vx[3 * k + 1] * m[a][1] + vx[3 * k + 2] * m[a][2]
                                       + vv[3 * k] * m[a][3] + vv[3 * k + 1] * m[a][4] + vv[3 * k + 2] * m[a][5];
        }
    }

    // ---- direct gravity, src/forces.c:266-433
    static const int order[NPL] = {B_PLU, B_MOO, B_MAR, B_MER, B_NEP, B_URA, B_EAR, B_VEN, B_SAT, B_JUP, B_SUN};
    const int na = e.n_ast();
    if (o.forces & (F_SUN | F_PLANETS | F_AST)) {
        for (int k = 0; k < NPL + na; k++) {
            int b = k >= na ? order[k - na] : k + NPL;
            if (b == B_SUN && !(o.forces & F_SUN)) continue;
            if (b > B_SUN && b < NPL && !(o.forces & F_PLANETS)) continue;
            if (b >= NPL && !(o.forces & F_AST)) continue;
            for (int j = 0; j < n_real; j++) {
                T dx = x[3 * j] + osub(xo[0], BX(b, 0));
                T dy = x[3 * j + 1] + osub(xo[1], BX(b, 1));
                T dz = x[3 * j + 2] + osub(xo[2], BX(b, 2));
                T r2 = dx * dx + dy * dy + dz * dz;
                T r = sqrt(r2);
                T pre = GM(b) / (r * r * r);
                acc[3 * j] -= pre * dx;
                acc[3 * j + 1] -= pre * dy;
                acc[3 * j + 2] -= pre * dz;
            }
        }
    }
    // variational direct terms from every body whatever the individual gravity
    // bits say, but only when the direct routine runs at all (src/forces.c:145-147, 352-432)
    if (n_var > 0 && (o.forces & (F_SUN | F_PLANETS | F_AST))) {
        for (int k = 0; k < NPL + na; k++) {
            int b = k >= na ? order[k - na] : k + NPL;
            for (int j = 0; j < n_real; j++) {
                if (vars[(size_t)j].empty()) continue;
                T dx = x[3 * j] + osub(xo[0], BX(b, 0));
                T dy = x[3 * j + 1] + osub(xo[1], BX(b, 1));
                T dz = x[3 * j + 2] + osub(xo[2], BX(b, 2));
                T r2 = dx * dx + dy * dy + dz * dz;
                T r = sqrt(r2);
                T r3i = 1. / (r2 * r);
                T r5i = 3. * r3i / r2;
                T mxx = dx * dx * r5i - r3i, myy = dy * dy * r5i - r3i, mzz = dz * dz * r5i - r3i;
                T mxy = dx * dy * r5i, mxz = dx * dz * r5i, myz = dy * dz * r5i;
                for (int q : vars[(size_t)j]) {
                    T ddx = vx[3 * q], ddy = vx[3 * q + 1], ddz = vx[3 * q + 2];
                    avar[3 * q] += GM(b) * (ddx * mxx + ddy * mxy + ddz * mxz);
                    avar[3 * q + 1] += GM(b) * (ddx * mxy + ddy * myy + ddz * myz);
                    avar[3 * q + 2] += GM(b) * (ddx * mxz + ddy * myz + ddz * mzz);
                }
            }
        }
    }
    // geocentric indirect term, src/forces.c:157-172
    if (o.geocentric == 1)
        for (int j = 0; j < n_real; j++)
            for (int a = 0; a < 3; a++) acc[3 * j + a] -= ao[a];
    return OK;
}

/* ---------------------------------------------------------------- IAS15 */
struct IasConst {
    double h[8];
    double rr[8][8];     // rr[n][j] = h[n] - h[j]
    double c[7][7];      // b_k += c[j][k] * dg_j  (k < j)
    double d[7][7];      // g_j = b_j + sum_{k>j} d[j][k] b_k
};

/* The Gauss-Radau nodes on [0,1] with h0 = 0: the 7 roots of
 * (P7 + P8)/(1 + x) on (-1, 1), mapped by h = (1+x)/2, bracketed on a fine
 * grid and refined by bisection in long double; the g<->b transforms follow
 * from expanding the Newton basis h*prod(h - h_i) in monomials and inverting
 * the triangular map. */
static long double radau_f(long double x) {
    long double p0 = 1, p1 = x, p7 = 0;
    for (int n = 1; n < 8; n++) {
        long double p2 = ((2 * n + 1) * x * p1 - n * p0) / (n + 1);
        p0 = p1; p1 = p2;
        if (n + 1 == 7) p7 = p1;
    }
    return (p7 + p1) / (1 + x);
}
static IasConst make_constants() {
    IasConst C;
    typedef long double L;
    L roots[7];
    int nr = 0;
    const int M = 20000;
    L xa = -1 + 1e-9L, fa = radau_f(xa);
    for (int i = 1; i <= M && nr < 7; i++) {
        L xb = -1 + 2.0L * i / M - (i == M ? 1e-9L : 0), fb = radau_f(xb);
        if ((fa < 0) != (fb < 0)) {
            L lo = xa, hi = xb, flo = fa;
            for (int it = 0; it < 200; it++) {
                L mid = (lo + hi) / 2, fm = radau_f(mid);
                if ((fm < 0) == (flo < 0)) { lo = mid; flo = fm; } else hi = mid;
            }
            roots[nr++] = (lo + hi) / 2;
        }
        xa = xb; fa = fb;
    }
    for (int i = 0; i < 7; i++)
        for (int j = i + 1; j < 7; j++)
            if (roots[j] < roots[i]) { L t = roots[i]; roots[i] = roots[j]; roots[j] = t; }
    L h[8];
    h[0] = 0;
    for (int k = 0; k < 7; k++) h[k + 1] = (1 + roots[k]) / 2;
    for (int n = 0; n < 8; n++) { C.h[n] = (double)h[n]; for (int j = 0; j < 8; j++) C.rr[n][j] = (double)(h[n] - h[j]); }
    L cm[7][7] = {{0}};
    for (int j = 0; j < 7; j++) {
        L poly[8] = {1};
        int deg = 0;
        for (int i = 1; i <= j; i++) {
            L nw[8] = {0};
            for (int q = 0; q <= deg; q++) { nw[q + 1] += poly[q]; nw[q] -= poly[q] * h[i]; }
            deg++;
            for (int q = 0; q <= deg; q++) poly[q] = nw[q];
        }
        for (int q = 0; q <= deg; q++) cm[j][q] = poly[q];   // b_q += cm[j][q] g_j
    }
    // D = C^-1 (upper triangular with unit diagonal in the (k, j) orientation)
    L dm[7][7] = {{0}};
    for (int j = 6; j >= 0; j--) {
        dm[j][j] = 1;
        for (int k = j + 1; k < 7; k++) {
            L s = 0;
            for (int q = j; q < k; q++) s += dm[j][q] * cm[k][q];
            dm[j][k] = -s;
        }
    }
    for (int j = 0; j < 7; j++) for (int k = 0; k < 7; k++) { C.c[j][k] = (double)cm[j][k]; C.d[j][k] = (double)dm[j][k]; }
    return C;
}
static const IasConst& K() { static IasConst k = make_constants(); return k; }

struct IasOpts { double epsilon, min_dt; int max_steps; int max_iter; double dt_floor; };
struct IasStats { long long accepted, rejected, evals, iterations; int status; };

template <class T>
struct ForceFn {
    virtual int eval(T t, double dt_sign, const T* x, const T* v, T* a) = 0;
    virtual ~ForceFn() {}
};

/* IAS15 state for N particles of which the first n_real are real (error
 * measures use only those). */
template <class T>
struct Ias15 {
    int N, n_real;
    T t, tc;                                   // time and its compensation
    T dt, dt_last_success;
    std::vector<T> x0, v0, a0, xc, vc, at, x, v;
    std::vector<T> b[7], g[7], e[7], br[7], er[7];
    Ias15(int N_, int nr) : N(N_), n_real(nr), t(0.0), tc(0.0), dt(0.0), dt_last_success(0.0) {
        size_t n3 = 3 * (size_t)N;
        x0.assign(n3, T(0.0)); v0 = x0; a0 = x0; xc = x0; vc = x0; at = x0; x = x0; v = x0;
        for (int k = 0; k < 7; k++) { b[k] = x0; g[k] = x0; e[k] = x0; br[k] = x0; er[k] = x0; }
    }
    void predict_next(T ratio) {
        const size_t n3 = 3 * (size_t)N;
        if (ratio > T(20.0)) {
            for (int k = 0; k < 7; k++) for (size_t i = 0; i < n3; i++) { e[k][i] = 0.0; b[k][i] = 0.0; }
            return;
        }
        T q[8];
        q[1] = ratio;
        for (int k = 2; k < 8; k++) q[k] = q[k - 1] * ratio;
        // shift of the old step's acceleration polynomial to the new step:
        // e_j = q^(j+1) * sum_{k>=j} binom(k+1, j+1) b_k
        static const double binom[8][8] = {
            {1, 0, 0, 0, 0, 0, 0, 0}, {1, 1, 0, 0, 0, 0, 0, 0}, {1, 2, 1, 0, 0, 0, 0, 0}, {1, 3, 3, 1, 0, 0, 0, 0},
            {1, 4, 6, 4, 1, 0, 0, 0}, {1, 5, 10, 10, 5, 1, 0, 0}, {1, 6, 15, 20, 15, 6, 1, 0}, {1, 7, 21, 35, 35, 21, 7, 1}};
        for (size_t i = 0; i < n3; i++) {
            T be[7];
            for (int k = 0; k < 7; k++) be[k] = br[k][i] - er[k][i];
            for (int j = 0; j < 7; j++) {
                T s = 0.0;
                for (int k = 6; k >= j; k--) s += br[k][i] * binom[k + 1][j + 1];
                e[j][i] = q[j + 1] * s;
            }
            for (int k = 0; k < 7; k++) b[k][i] = e[k][i] + be[k];
        }
    }
    /* One attempted step of size `h` (sign = direction).  Returns 1 accepted,
     * 0 rejected, <0 force error. */
    int step(ForceFn<T>& F, T hstep, const IasOpts& o, IasStats& st, T* dt_new_out, bool cut = false) {
        const IasConst& C = K();
        const size_t n3 = 3 * (size_t)N, nr3 = 3 * (size_t)n_real;
        const double sgn = to_double(hstep) >= 0 ? 1.0 : -1.0;
        int f = F.eval(t, sgn, x0.data(), v0.data(), a0.data());
        st.evals++;
        if (f != OK) return -f;
        for (size_t i = 0; i < n3; i++) {
            for (int j = 0; j < 7; j++) {
                T s = b[j][i];
                for (int k = j + 1; k < 7; k++) s += b[k][i] * C.d[j][k];
                g[j][i] = s;
            }
        }
        T pc_err = 1e300, pc_last = 2.0;
        int iters = 0;
        while (true) {
            if (pc_err < T(1e-16)) break;
            if (iters > 2 && !(pc_err < pc_last)) break;
            if (iters >= o.max_iter) break;
            pc_last = pc_err;
            pc_err = 0.0;
            iters++;
            for (int n = 1; n < 8; n++) {
                const double hn = C.h[n];
                T sx[9], sv[8];
                sx[0] = hstep * hn;
                sx[1] = sx[0] * sx[0] / 2.;
                for (int k = 2; k < 9; k++) sx[k] = sx[k - 1] * (hn * (double)(k - 1) / (double)(k + 1));
                sv[0] = hstep * hn;
                for (int k = 1; k < 8; k++) sv[k] = sv[k - 1] * (hn * (double)k / (double)(k + 1));
                for (size_t i = 0; i < n3; i++) {
                    T px = sx[8] * b[6][i];
                    for (int k = 5; k >= 0; k--) px += sx[k + 2] * b[k][i];
                    px += sx[1] * a0[i];
                    px += sx[0] * v0[i];
                    x[i] = x0[i] + (px + xc[i]);
                    T pv = sv[7] * b[6][i];
                    for (int k = 5; k >= 0; k--) pv += sv[k + 1] * b[k][i];
                    pv += sv[0] * a0[i];
                    v[i] = v0[i] + (pv + vc[i]);
                }
                T tn = t + (tc + hstep * hn);
                f = F.eval(tn, sgn, x.data(), v.data(), at.data());
                st.evals++;
                if (f != OK) return -f;
                T maxa = 0.0, maxdb = 0.0;
                for (size_t i = 0; i < n3; i++) {
                    T gk = at[i] - a0[i];
                    T gn = gk / C.rr[n][0];
                    for (int j = 1; j < n; j++) gn = (gn - g[j - 1][i]) / C.rr[n][j];
                    T delta = gn - g[n - 1][i];
                    g[n - 1][i] = gn;
                    for (int k = 0; k < n - 1; k++) b[k][i] += delta * C.c[n - 1][k];
                    b[n - 1][i] += delta;
                    if (n == 7 && i < nr3) {
                        T aa = fabs(at[i]);
                        if (std::isnormal(to_double(aa)) && aa > maxa) maxa = aa;
                        T dd_ = fabs(delta);
                        if (std::isnormal(to_double(dd_)) && dd_ > maxdb) maxdb = dd_;
                    }
                }
                if (n == 7) pc_err = maxdb / maxa;
            }
        }
        st.iterations += iters;
        T dt_done = hstep;
        T dt_new = hstep;
        if (o.epsilon > 0.0) {
            T maxa = 0.0, maxb6 = 0.0;
            for (size_t i = 0; i < nr3; i++) {
                T aa = fabs(at[i]);
                if (std::isnormal(to_double(aa)) && aa > maxa) maxa = aa;
                T bb = fabs(b[6][i]);
                if (std::isnormal(to_double(bb)) && bb > maxb6) maxb6 = bb;
            }
            T err = maxb6 / maxa;
            const double safety = 0.25;
            if (std::isnormal(to_double(err))) dt_new = T(std::pow(o.epsilon / to_double(err), 1.0 / 7.0)) * dt_done;
            else dt_new = dt_done / safety;
            if (to_double(fabs(dt_new)) < o.min_dt) dt_new = T(std::copysign(o.min_dt, to_double(dt_new)));
            /* step underflow (an impact): stop, keeping the state of the step start.
             * Not on a step cut short to land on t_end: the proposal scales
             * with that short step and says nothing about the orbit. */
            if (!cut && o.dt_floor > 0.0 && to_double(fabs(dt_new)) < o.dt_floor) { *dt_new_out = dt_new; return 2; }
            T ratio = dt_new / dt_done;
            if (fabs(ratio) < T(safety)) {
                // rejected: re-predict from the last accepted step, or start from zero
                if (to_double(dt_last_success) != 0.0) predict_next(dt_new / dt_last_success);
                else for (int k = 0; k < 7; k++) for (size_t i = 0; i < n3; i++) { b[k][i] = 0.0; e[k][i] = 0.0; }
                *dt_new_out = dt_new;
                st.rejected++;
                return 0;
            }
            if (fabs(ratio) > T(1.0 / safety)) dt_new = dt_done / safety;
        }
        // accept: advance x0, v0 with compensated sums
        for (size_t i = 0; i < n3; i++) {
            T ix = b[6][i] / 72. + b[5][i] / 56. + b[4][i] / 42. + b[3][i] / 30. + b[2][i] / 20. + b[1][i] / 12. + b[0][i] / 6. + a0[i] / 2.;
            ix = ix * dt_done * dt_done + v0[i] * dt_done;
            T y = ix + xc[i];
            T s = x0[i] + y;
            xc[i] = y - (s - x0[i]);
            x0[i] = s;
            T iv = b[6][i] / 8. + b[5][i] / 7. + b[4][i] / 6. + b[3][i] / 5. + b[2][i] / 4. + b[1][i] / 3. + b[0][i] / 2. + a0[i];
            iv = iv * dt_done;
            y = iv + vc[i];
            s = v0[i] + y;
            vc[i] = y - (s - v0[i]);
            v0[i] = s;
        }
        {
            T y = dt_done + tc;
            T s = t + y;
            tc = y - (s - t);
            t = s;
        }
        dt_last_success = dt_done;
        for (int k = 0; k < 7; k++) { er[k] = e[k]; br[k] = b[k]; }
        predict_next(dt_new / dt_done);
        *dt_new_out = dt_new;
        st.accepted++;
        return 1;
    }
    /* Integrate to t_end exactly (last step shortened). */
    int integrate(ForceFn<T>& F, T t_end, const IasOpts& o, IasStats& st) {
        const double dir = to_double(t_end - t) >= 0 ? 1.0 : -1.0;
        if (to_double(dt) * dir <= 0) dt = T(std::fabs(to_double(dt)) * dir);
        long long steps = 0;
        while (to_double(t) != to_double(t_end)) {
            T rem = (t_end - t) - tc;
            bool last = false;
            T h = dt;
            if (to_double(fabs(dt)) >= to_double(fabs(rem))) { h = rem; last = true; }
            T dtn;
            int r = step(F, h, o, st, &dtn, last);
            if (r < 0) { st.status = 1; return -r; }
            if (r == 2) { st.status = 4; return 0; }
            dt = dtn;
            if (r == 1) {
                if (last) { t = t_end; tc = 0.0; }
                if (o.max_steps > 0 && ++steps >= o.max_steps && to_double(t) != to_double(t_end)) { st.status = 3; return 0; }
            }
        }
        st.status = 0;
        return 0;
    }
};

/* Force function over the oracle's own force model.  x/v hold the n_real real
 * particles first, then the n_var variational particles. */
template <class T>
struct OracleForces : ForceFn<T> {
    const Ephem* e; ForceOpts o; int n_real, n_var; std::vector<int> vtp; const double* params;
    int eval(T t, double, const T* x, const T* v, T* a) override {
        return forces<T>(*e, o, t, n_real, x, v, n_var, vtp.data(), x + 3 * n_real, v + 3 * n_real, params, a);
    }
};

typedef int (*orc_force_cb)(void* ctx, double t, double dt_sign, const double* x, const double* v, double* a);
struct CallbackForces : ForceFn<double> {
    orc_force_cb cb; void* ctx;
    int eval(double t, double s, const double* x, const double* v, double* a) override { return cb(ctx, t, s, x, v, a); }
};

}  // namespace

/* ========================================================================= C ABI */
extern "C" {

void* orc_ephem_load(const char* planets, const char* asteroids) { return ephem_load(planets, asteroids); }
void orc_ephem_free(void* h) {
    Ephem* e = (Ephem*)h;
    if (!e) return;
    delete e->pl; delete e->ast; delete e->pls; delete e;
}
int orc_n_bodies(void* h) { return NPL + ((Ephem*)h)->n_ast(); }
int orc_body(void* h, int i, double t, double* out) {
    Ephem* e = (Ephem*)h;
    if (i < 0 || i >= NPL + e->n_ast()) return i < NPL ? ERR_NEPHEM : ERR_NAST;
    return body_state<double>(*e, i, t, out);
}
void orc_time_bounds(void* h, double* tb, double* te) {
    Ephem* e = (Ephem*)h;
    double b = -INFINITY, en = INFINITY;
    if (e->pls) {
        for (auto& t : e->pls->targets) { if (t.beg > b) b = t.beg; if (t.end < en) en = t.end; }
    } else {
        b = e->pl->beg; en = e->pl->end;
    }
    if (e->ast) for (auto& t : e->ast->targets) { if (t.beg > b) b = t.beg; if (t.end < en) en = t.end; }
    *tb = b - e->jd_ref; *te = en - e->jd_ref;
}
/* out: AU EMRAT J2E J3E J4E J2SUN RE CLIGHT ASUN Re_eq Rs_eq c c2 1/c2 */
void orc_constants(void* h, double* out) {
    Ephem* e = (Ephem*)h;
    double v[14] = {e->AU, e->EMRAT, e->J2E, e->J3E, e->J4E, e->J2SUN, e->RE, e->CLIGHT, e->ASUN,
                    e->Re_eq, e->Rs_eq, e->c_AU_per_day, e->c_squared, e->over_c_squared};
    std::memcpy(out, v, sizeof(v));
}

static ForceOpts mkopts(int forces, int gr, int geo, const double* law) {
    ForceOpts o;
    o.forces = forces; o.gr_eih_sources = gr; o.geocentric = geo;
    o.alpha = law[0]; o.nk = law[1]; o.nm = law[2]; o.nn = law[3]; o.r0 = law[4];
    return o;
}

/* One force evaluation; law = {alpha, nk, nm, nn, r0}. acc: 3*(n_real+n_var). */
int orc_forces(void* h, int fbits, int gr_eih_sources, int geocentric, const double* law, double t,
               int n_real, const double* x, const double* v, int n_var, const int* vtp, const double* vx,
               const double* vv, const double* params, double* acc) {
    ForceOpts o = mkopts(fbits, gr_eih_sources, geocentric, law);
    return forces<double>(*(Ephem*)h, o, t, n_real, x, v, n_var, vtp, vx, vv, params, acc);
}

/* Same in double-double: inputs are doubles, acc_hi/acc_lo receive the parts. */
int orc_forces_dd(void* h, int fbits, int gr_eih_sources, int geocentric, const double* law, double t,
                  int n_real, const double* x, const double* v, int n_var, const int* vtp, const double* vx,
                  const double* vv, const double* params, double* acc_hi, double* acc_lo) {
    ForceOpts o = mkopts(fbits, gr_eih_sources, geocentric, law);
    std::vector<dd> X(x, x + 3 * n_real), V(v, v + 3 * n_real), VX(vx, vx + 3 * n_var), VV(vv, vv + 3 * n_var);
    std::vector<dd> A(3 * (size_t)(n_real + n_var));
    int r = forces<dd>(*(Ephem*)h, o, dd(t), n_real, X.data(), V.data(), n_var, vtp, VX.data(), VV.data(), params, A.data());
    for (size_t i = 0; i < A.size(); i++) { acc_hi[i] = A[i].hi; acc_lo[i] = A[i].lo; }
    return r;
}

/* Operation counts of one force evaluation for a single real particle (with
 * its n_var variational particles), including the evaluation of every body
 * at that particle's time.  out[0..4]: add, mul, div, sqrt, pow of the
 * particle-dependent work and the body states; out[5..9]: the body-state part
 * of out[0..4]; out[10..14]: force-term work that does not depend on the
 * particle, tallied apart. */
int orc_count_ops(void* h, int fbits, int gr_eih_sources, int geocentric, const double* law, double t,
                  const double* x, const double* v, int n_var, const double* vx, const double* vv,
                  const double* params, long long* out) {
    ForceOpts o = mkopts(fbits, gr_eih_sources, geocentric, law);
    std::vector<cnt> X(x, x + 3), V(v, v + 3), VX(vx, vx + 3 * n_var), VV(vv, vv + 3 * n_var);
    std::vector<cnt> A(3 * (size_t)(1 + n_var));
    std::vector<int> vtp((size_t)n_var, 0);
    g_tally = OpTally{0, 0, 0, 0, 0};
    g_tally_bodies = OpTally{0, 0, 0, 0, 0};
    g_tally_shared = OpTally{0, 0, 0, 0, 0};
    int r = forces<cnt>(*(Ephem*)h, o, cnt(t), 1, X.data(), V.data(), n_var, vtp.data(), VX.data(), VV.data(), params, A.data());
    out[0] = g_tally.add; out[1] = g_tally.mul; out[2] = g_tally.div; out[3] = g_tally.sqrt; out[4] = g_tally.fn;
    /* out[5..9]: the part of it that forms the body states (all bodies at t) */
    out[5] = g_tally_bodies.add; out[6] = g_tally_bodies.mul; out[7] = g_tally_bodies.div;
    out[8] = g_tally_bodies.sqrt; out[9] = g_tally_bodies.fn;
    /* out[10..14]: force-term work that does not depend on the particle
     * (origin-minus-body offsets, EIH source-source sums), not in out[0..4] */
    out[10] = g_tally_shared.add; out[11] = g_tally_shared.mul; out[12] = g_tally_shared.div;
    out[13] = g_tally_shared.sqrt; out[14] = g_tally_shared.fn;
    return r;
}

/* Gauss-Radau constants as computed here (for comparison with the product's). */
void orc_ias15_constants(double* h8, double* c49, double* d49) {
    const IasConst& C = K();
    for (int i = 0; i < 8; i++) h8[i] = C.h[i];
    for (int j = 0; j < 7; j++) for (int k = 0; k < 7; k++) { c49[7 * j + k] = C.c[j][k]; d49[7 * j + k] = C.d[j][k]; }
}

/* Integrate ONE simulation (shared step) of n_real real + n_var variational
 * particles from t0 to t_end.  state: 6*(n_real+n_var) (x,y,z,vx,vy,vz per
 * particle, real first), overwritten.  stats: accepted, rejected, evals,
 * iterations, status.  use_dd=1 runs the double-double oracle. */
int orc_integrate(void* h, int fbits, int gr_eih_sources, int geocentric, const double* law, double t0,
                  double t_end, int n_real, int n_var, const int* vtp, double* state, const double* params,
                  double epsilon, double min_dt, double dt0, int max_steps, double dt_floor, int use_dd, long long* stats,
                  double* t_out, double* dt_out) {
    const int N = n_real + n_var;
    IasOpts io{epsilon, min_dt, max_steps, 12, dt_floor};
    IasStats st{0, 0, 0, 0, 0};
    int r;
    if (!use_dd) {
        OracleForces<double> F;
        F.e = (Ephem*)h; F.o = mkopts(fbits, gr_eih_sources, geocentric, law); F.n_real = n_real; F.n_var = n_var;
        F.vtp.assign(vtp, vtp + n_var); F.params = params;
        Ias15<double> I(N, n_real);
        for (int i = 0; i < N; i++) for (int k = 0; k < 3; k++) { I.x0[3 * i + k] = state[6 * i + k]; I.v0[3 * i + k] = state[6 * i + 3 + k]; }
        I.t = t0; I.dt = dt0;
        r = I.integrate(F, t_end, io, st);
        for (int i = 0; i < N; i++) for (int k = 0; k < 3; k++) { state[6 * i + k] = I.x0[3 * i + k] + I.xc[3 * i + k]; state[6 * i + 3 + k] = I.v0[3 * i + k] + I.vc[3 * i + k]; }
        if (t_out) *t_out = I.t;
        if (dt_out) *dt_out = I.dt;
    } else {
        OracleForces<dd> F;
        F.e = (Ephem*)h; F.o = mkopts(fbits, gr_eih_sources, geocentric, law); F.n_real = n_real; F.n_var = n_var;
        F.vtp.assign(vtp, vtp + n_var); F.params = params;
        Ias15<dd> I(N, n_real);
        for (int i = 0; i < N; i++) for (int k = 0; k < 3; k++) { I.x0[3 * i + k] = state[6 * i + k]; I.v0[3 * i + k] = state[6 * i + 3 + k]; }
        I.t = t0; I.dt = dt0;
        r = I.integrate(F, dd(t_end), io, st);
        for (int i = 0; i < N; i++) for (int k = 0; k < 3; k++) {
            state[6 * i + k] = to_double(I.x0[3 * i + k] + I.xc[3 * i + k]);
            state[6 * i + 3 + k] = to_double(I.v0[3 * i + k] + I.vc[3 * i + k]);
        }
        if (t_out) *t_out = to_double(I.t);
        if (dt_out) *dt_out = to_double(I.dt);
    }
    if (stats) { stats[0] = st.accepted; stats[1] = st.rejected; stats[2] = st.evals; stats[3] = st.iterations; stats[4] = st.status; }
    return r;
}

/* IAS15 over an arbitrary force callback (double only), e.g. the reference's
 * own assist_additional_forces through oracle/_ref's harness. */
int orc_integrate_cb(orc_force_cb cb, void* ctx, double t0, double t_end, int N, int n_real, double* state,
                     double epsilon, double min_dt, double dt0, int max_steps, long long* stats) {
    CallbackForces F;
    F.cb = cb; F.ctx = ctx;
    IasOpts io{epsilon, min_dt, max_steps, 12, 0.0};
    IasStats st{0, 0, 0, 0, 0};
    Ias15<double> I(N, n_real);
    for (int i = 0; i < N; i++) for (int k = 0; k < 3; k++) { I.x0[3 * i + k] = state[6 * i + k]; I.v0[3 * i + k] = state[6 * i + 3 + k]; }
    I.t = t0; I.dt = dt0;
    int r = I.integrate(F, t_end, io, st);
    for (int i = 0; i < N; i++) for (int k = 0; k < 3; k++) { state[6 * i + k] = I.x0[3 * i + k] + I.xc[3 * i + k]; state[6 * i + 3 + k] = I.v0[3 * i + k] + I.vc[3 * i + k]; }
    if (stats) { stats[0] = st.accepted; stats[1] = st.rejected; stats[2] = st.evals; stats[3] = st.iterations; stats[4] = st.status; }
    return r;
}

/* Warm-start ceiling study (test infrastructure: what any predictor of
 * IAS15's b can save).  Particles are integrated in shared-step groups of
 * `group` consecutive particles (group = 1: independent steps; the group's
 * error and convergence measures are maxima over its members, as in a
 * kernel whose members share each step), each group from t0[first] to
 * t_end[first].  At every accepted step the step is replayed from its saved
 * start with the predictor's b replaced by b_conv (1 + rel_err[k] u), u
 * uniform in [-1, 1] per coefficient (seeded), for each of the n_err
 * relative errors (0: the converged b itself), and the replay's
 * predictor-corrector iterations are tallied.  hist: (1 + n_err) rows of 13
 * counts of accepted steps by iterations, row 0 the plain predictor's. */
int orc_warm_start_study(void* h, int fbits, int gr_eih_sources, int geocentric, const double* law, int n,
                         int group, const double* t0, const double* t_end, const double* state, const double* params,
                         double epsilon, double dt0, double dt_floor, int threads, int n_err, const double* rel_err,
                         unsigned long long seed, long long* hist) {
    if (group < 1 || n_err < 0 || n_err > 16) return -1;
    const int ng = (n + group - 1) / group;
    std::atomic<int> next(0);
    std::vector<long long> H((size_t)(1 + n_err) * 13 * (size_t)(threads > 0 ? threads : 1), 0);
    auto work = [&](int tid) {
        long long* Ht = H.data() + (size_t)tid * (1 + n_err) * 13;
        OracleForces<double> F;
        F.e = (Ephem*)h; F.o = mkopts(fbits, gr_eih_sources, geocentric, law); F.n_var = 0;
        IasOpts io{epsilon, 0.0, 0, 12, dt_floor};
        uint64_t rs = seed * 0x9E3779B97F4A7C15ull + 1 + (uint64_t)tid;
        auto uni = [&]() {     /* xorshift64*, uniform in [-1, 1] */
            rs ^= rs >> 12; rs ^= rs << 25; rs ^= rs >> 27;
            return (double)((rs * 0x2545F4914F6CDD1Dull) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        };
        while (true) {
            const int g = next.fetch_add(1);
            if (g >= ng) break;
            const int i0 = g * group, m = std::min(group, n - i0);
            F.n_real = m;
            F.vtp.clear();
            std::vector<double> prm;
            F.params = nullptr;
            if (params) { prm.assign(params + 3 * (size_t)i0, params + 3 * (size_t)(i0 + m)); F.params = prm.data(); }
            Ias15<double> I(m, m);
            for (int j = 0; j < m; j++)
                for (int k = 0; k < 3; k++) {
                    I.x0[3 * j + k] = state[6 * (size_t)(i0 + j) + k];
                    I.v0[3 * j + k] = state[6 * (size_t)(i0 + j) + 3 + k];
                }
            I.t = t0[i0]; I.dt = dt0;
            const double te = t_end[i0];
            const double dir = te - I.t >= 0 ? 1.0 : -1.0;
            if (I.dt * dir <= 0) I.dt = std::fabs(I.dt) * dir;
            IasStats st{0, 0, 0, 0, 0};
            while (I.t != te) {
                const double rem = (te - I.t) - I.tc;
                bool last = false;
                double hs = I.dt;
                if (std::fabs(I.dt) >= std::fabs(rem)) { hs = rem; last = true; }
                Ias15<double> S0 = I;
                const long long it0 = st.iterations;
                double dtn;
                const int r = I.step(F, hs, io, st, &dtn, last);
                if (r < 0 || r == 2) break;
                if (r == 1) {
                    Ht[std::min<long long>(st.iterations - it0, 12)]++;
                    for (int q = 0; q < n_err; q++) {
                        Ias15<double> R = S0;
                        for (int k = 0; k < 7; k++)
                            for (size_t c = 0; c < R.b[k].size(); c++) R.b[k][c] = I.br[k][c] * (1.0 + rel_err[q] * uni());
                        IasStats sr{0, 0, 0, 0, 0};
                        double dtr;
                        R.step(F, hs, io, sr, &dtr, last);
                        Ht[(size_t)(1 + q) * 13 + std::min<long long>(sr.iterations, 12)]++;
                    }
                }
                I.dt = dtn;
                if (r == 1 && last) { I.t = te; I.tc = 0.0; }
            }
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int k = 1; k < threads; k++) pool.emplace_back(work, k);
    work(0);
    for (auto& th : pool) th.join();
    for (size_t k = 0; k < (size_t)(1 + n_err) * 13; k++) {
        hist[k] = 0;
        for (int t = 0; t < threads; t++) hist[k] += H[(size_t)t * (1 + n_err) * 13 + k];
    }
    return 0;
}

/* Batched independent particles: particle i (with n_var_each variational
 * particles, 0 or 6) is its own simulation from t0[i] to t_end[i].
 * state: n*6; var_state: n*n_var_each*6; params: n*3 rows for the real
 * particle (variational rows get dA = 0) or NULL.  Runs on `threads` host
 * threads.  stats: sum of accepted, rejected, evals, iterations. */
int orc_integrate_batch(void* h, int fbits, int gr_eih_sources, int geocentric, const double* law, int n,
                        const double* t0, const double* t_end, double* state, const double* params,
                        int n_var_each, double* var_state, int* status, double epsilon, double min_dt,
                        double dt0, int max_steps, double dt_floor, int threads, long long* stats) {
    std::atomic<int> next(0);
    std::atomic<long long> acc(0), rej(0), ev(0), it(0);
    auto work = [&]() {
        OracleForces<double> F;
        F.e = (Ephem*)h; F.o = mkopts(fbits, gr_eih_sources, geocentric, law); F.n_real = 1; F.n_var = n_var_each;
        F.vtp.assign((size_t)n_var_each, 0);
        std::vector<double> prm(3 * (size_t)(1 + n_var_each), 0.0);
        IasOpts io{epsilon, min_dt, max_steps, 12, dt_floor};
        while (true) {
            int i = next.fetch_add(1);
            if (i >= n) break;
            F.params = nullptr;
            if (params) { for (int k = 0; k < 3; k++) prm[k] = params[3 * (size_t)i + k]; F.params = prm.data(); }
            Ias15<double> I(1 + n_var_each, 1);
            for (int k = 0; k < 3; k++) { I.x0[k] = state[6 * (size_t)i + k]; I.v0[k] = state[6 * (size_t)i + 3 + k]; }
            for (int q = 0; q < n_var_each; q++)
                for (int k = 0; k < 3; k++) {
                    I.x0[3 * (1 + q) + k] = var_state[(size_t)(i * n_var_each + q) * 6 + k];
                    I.v0[3 * (1 + q) + k] = var_state[(size_t)(i * n_var_each + q) * 6 + 3 + k];
                }
            I.t = t0[i]; I.dt = dt0;
            IasStats st{0, 0, 0, 0, 0};
            int r = I.integrate(F, t_end[i], io, st);
            for (int k = 0; k < 3; k++) { state[6 * (size_t)i + k] = I.x0[k] + I.xc[k]; state[6 * (size_t)i + 3 + k] = I.v0[k] + I.vc[k]; }
            for (int q = 0; q < n_var_each; q++)
                for (int k = 0; k < 3; k++) {
                    var_state[(size_t)(i * n_var_each + q) * 6 + k] = I.x0[3 * (1 + q) + k] + I.xc[3 * (1 + q) + k];
                    var_state[(size_t)(i * n_var_each + q) * 6 + 3 + k] = I.v0[3 * (1 + q) + k] + I.vc[3 * (1 + q) + k];
                }
            if (status) status[i] = r != 0 ? 1 : st.status;
            acc += st.accepted; rej += st.rejected; ev += st.evals; it += st.iterations;
        }
    };
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int k = 1; k < threads; k++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    if (stats) { stats[0] = acc; stats[1] = rej; stats[2] = ev; stats[3] = it; }
    return 0;
}

}  // extern "C"
