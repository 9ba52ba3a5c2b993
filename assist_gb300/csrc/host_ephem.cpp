/*
 * host_ephem.cpp -- ephemeris front door: format detection, discovery, the
 * .440 and SPK loaders, and the device images the kernels read.
 *
 * Behaviour follows ASSIST's front door (src/assist.c:62-377):
 *   - detection: "DAF/SPK " at offset 0 -> SPK; otherwise plausible 6-byte
 *     constant names at 0x00FC -> .440/.441 (src/assist.c:66-135);
 *   - discovery under ASSIST_DIR in the order de441.bsp, de440.bsp,
 *     linux_m13000p17000.441, linux_p1550p2650.440 (src/assist.c:137-154);
 *   - .440 header fields, constant table and GM values as read by
 *     src/ascii_ephem.c:105-252 (EMRAT split of GMB into Earth and Moon);
 *   - SPK summaries collected per target, segment directories, and the
 *     asteroid GMs from the .440 "MAnnnn" constants (src/assist.c:311-333).
 *   - planets from an SPK (.bsp) file: the constants and GMs of the
 *     comment area (src/spk.c:49-110, 695-800), masses joined to targets
 *     by name with the Earth/Moon split of GMB (src/spk.c:137-200), target
 *     indices of the eleven bodies and of the Earth-Moon barycentre
 *     (src/assist.c:252-292).
 * The parsed files are copied to device memory once; the kernels read the
 * same words ASSIST reads through its mmap.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fcntl.h>
#include <string>
#include <unistd.h>
#include <vector>

#include "../../include/assist.h"
#include "internal.h"

/* ------------------------------------------------------------ the objects
 * behind struct assist_ephem's opaque pointers */
struct ascii_s {
    double beg, end, inc, cau, cem;
    int num, ver;
    int off[15], ncf[15], niv[15], ncm[15];
    size_t rec;                          /* doubles per record */
    std::vector<double> data;            /* the file as doubles */
    std::vector<std::string> names;
    std::vector<double> con;
    double mass[ASSIST_BODY_NPLANETS];
    double J2E, J3E, J4E, J2SUN, AU, RE, CLIGHT, ASUN;
    double* d_data = nullptr;
    DevEphem* d_view = nullptr;      /* device copy of the last view handed to kernels */
    DevEphem h_view;                 /* host copy of *d_view */
    bool find(const char* name, double* out) const {
        char key[7] = "      ";
        for (int i = 0; i < 6 && name[i]; i++) key[i] = name[i];
        for (size_t p = 0; p < names.size(); p++)
            if (std::memcmp(names[p].data(), key, 6) == 0) { *out = con[p]; return true; }
        *out = 0.0;
        return false;
    }
};

struct spk_target_h {
    int code, cen;
    double mass, beg, end, res;
    std::vector<int> one, two;
};
struct spk_s {
    std::vector<spk_target_h> targets;
    std::vector<double> data;
    std::vector<AgSpkSeg> segs;
    std::vector<AgRecMeta> meta;
    std::vector<int> seg0;
    std::string comments;            /* comment area, NUL -> newline */
    double* d_data = nullptr;
    AgSpkSeg* d_segs = nullptr;
    AgRecMeta* d_meta = nullptr;
    DevEphem* d_view = nullptr;      /* planets files: device copy of the last view */
    DevEphem h_view;
};

static bool read_file(const char* path, std::vector<unsigned char>& out) {
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
template <class X> static X get(const std::vector<unsigned char>& b, size_t off) {
    X x;
    std::memcpy(&x, b.data() + off, sizeof(X));
    return x;
}

/* ---------------------------------------------------------------- detection */
extern "C" int assist_detect_ascii_bin_signature(int fd) {
    char names[18];
    if (lseek(fd, 0x00FC, SEEK_SET) != 0x00FC) return 0;
    if (read(fd, names, sizeof(names)) != (ssize_t)sizeof(names)) return 0;
    int valid = 0;
    for (int i = 0; i < 3; i++) {
        const unsigned char* nm = (const unsigned char*)names + 6 * i;
        const bool alpha0 = (nm[0] >= 'A' && nm[0] <= 'Z') || (nm[0] >= 'a' && nm[0] <= 'z');
        if (!alpha0) continue;
        int alnum = 0;
        bool ok = true;
        for (int j = 0; j < 6; j++) {
            const unsigned char ch = nm[j];
            if ((ch >= 'A' && ch <= 'Z') || (ch >= 'a' && ch <= 'z') || (ch >= '0' && ch <= '9')) alnum++;
            else if (ch == ' ' || ch == '\0') { /* padding */ }
            else { ok = false; break; }
        }
        if (ok && alnum >= 2) valid++;
    }
    return valid >= 2;
}

extern "C" ephemeris_file_format_t assist_detect_ephemeris_file_format(int fd) {
    char buf[1024];
    lseek(fd, 0, SEEK_SET);
    ssize_t n = read(fd, buf, sizeof(buf));
    if (n <= 0) return FILE_FORMAT_UNKNOWN;
    if (n >= 8 && std::strncmp(buf, "DAF/SPK ", 8) == 0) return FILE_FORMAT_VALID_BSP;
    if (assist_detect_ascii_bin_signature(fd)) {
        lseek(fd, 0, SEEK_SET);
        return FILE_FORMAT_ASCII_BIN;
    }
    return FILE_FORMAT_UNKNOWN;
}

extern "C" int assist_discover_planets_path(char* out_path, size_t out_size, const char* assist_dir) {
    if (!out_path || out_size == 0 || !assist_dir) return 0;
    static const char* cand[] = {"/data/de441.bsp", "/data/de440.bsp", "/data/linux_m13000p17000.441",
                                 "/data/linux_p1550p2650.440"};
    for (const char* c : cand) {
        std::snprintf(out_path, out_size, "%s%s", assist_dir, c);
        if (access(out_path, R_OK) == 0) return 1;
    }
    return 0;
}

/* ---------------------------------------------------------------- loaders */
static ascii_s* ascii_load(const char* path) {
    std::vector<unsigned char> b;
    if (!read_file(path, b) || b.size() < 0x0B28 + 24) return nullptr;
    ascii_s* a = new ascii_s();
    std::memset(&a->h_view, 0, sizeof(a->h_view));
    size_t o = 0x0A5C;
    a->beg = get<double>(b, o); a->end = get<double>(b, o + 8); a->inc = get<double>(b, o + 16);
    a->num = get<int32_t>(b, o + 24); a->cau = get<double>(b, o + 28); a->cem = get<double>(b, o + 36);
    o += 44;
    for (int p = 0; p < 15; p++) a->ncm[p] = 3;
    a->ncm[11] = 2; a->ncm[14] = 1;
    for (int p = 0; p < 12; p++, o += 12) {
        a->off[p] = get<int32_t>(b, o); a->ncf[p] = get<int32_t>(b, o + 4); a->niv[p] = get<int32_t>(b, o + 8);
    }
    a->ver = get<int32_t>(b, o); o += 4;
    a->off[12] = get<int32_t>(b, o); a->ncf[12] = get<int32_t>(b, o + 4); a->niv[12] = get<int32_t>(b, o + 8);
    if (a->num < 0 || a->num > 100000 || !(a->inc > 0)) { delete a; return nullptr; }
    size_t tail = 0x0B28 + 6 * (size_t)(a->num > 400 ? a->num - 400 : 0);
    if (tail + 24 > b.size()) { delete a; return nullptr; }
    for (int p = 0; p < a->num; p++) {
        size_t no = p < 400 ? 0x00FC + 6 * (size_t)p : 0x0B28 + 6 * (size_t)(p - 400);
        a->names.emplace_back((const char*)b.data() + no, 6);
    }
    o = tail;
    for (int p = 13; p < 15; p++, o += 12) {
        a->off[p] = get<int32_t>(b, o); a->ncf[p] = get<int32_t>(b, o + 4); a->niv[p] = get<int32_t>(b, o + 8);
    }
    size_t rec = 2;
    for (int p = 0; p < 15; p++) {
        a->off[p] -= 1;
        if (a->ncf[p] < 0 || a->niv[p] < 0 || a->ncf[p] > AG_MAX_NCF) { delete a; return nullptr; }
        rec += (size_t)a->ncf[p] * a->niv[p] * a->ncm[p];
    }
    a->rec = rec;
    if (b.size() < 2 * rec * 8) { delete a; return nullptr; }
    for (int p = 0; p < 11; p++)
        if (a->off[p] < 2 || (size_t)a->off[p] + (size_t)a->ncf[p] * a->niv[p] * 3 > rec || a->ncf[p] < 2 || a->niv[p] < 1) {
            delete a; return nullptr;
        }
    a->data.resize(b.size() / 8);
    std::memcpy(a->data.data(), b.data(), a->data.size() * 8);
    for (int p = 0; p < a->num; p++) a->con.push_back(get<double>(b, rec * 8 + 8 * (size_t)p));
    double emrat = 0, gmb = 0;
    a->find("GMS", &a->mass[ASSIST_BODY_SUN]); a->find("GM1", &a->mass[ASSIST_BODY_MERCURY]);
    a->find("GM2", &a->mass[ASSIST_BODY_VENUS]);
    a->find("EMRAT", &emrat); a->find("GMB", &gmb);
    a->mass[ASSIST_BODY_EARTH] = (emrat / (1. + emrat)) * gmb;
    a->mass[ASSIST_BODY_MOON] = 1. / (1 + emrat) * gmb;
    a->find("GM4", &a->mass[ASSIST_BODY_MARS]); a->find("GM5", &a->mass[ASSIST_BODY_JUPITER]);
    a->find("GM6", &a->mass[ASSIST_BODY_SATURN]); a->find("GM7", &a->mass[ASSIST_BODY_URANUS]);
    a->find("GM8", &a->mass[ASSIST_BODY_NEPTUNE]); a->find("GM9", &a->mass[ASSIST_BODY_PLUTO]);
    a->find("J2E", &a->J2E); a->find("J3E", &a->J3E); a->find("J4E", &a->J4E); a->find("J2SUN", &a->J2SUN);
    a->find("AU", &a->AU); a->find("RE", &a->RE); a->find("CLIGHT", &a->CLIGHT); a->find("ASUN", &a->ASUN);
    return a;
}

/* The device copy of the .440 image, made on first device use (loading and
 * validating a file is host work only). */
static int ascii_upload(ascii_s* a) {
    if (a->d_data) return 0;
    /* 64 bytes of padding: a record staged by a bulk copy is read from its
     * address rounded down to 16 bytes, for its length rounded up */
    if (ag_cuda_check(cudaMalloc(&a->d_data, a->data.size() * 8 + 64), "cudaMalloc(.440 records)") ||
        ag_cuda_check(cudaMemcpy(a->d_data, a->data.data(), a->data.size() * 8, cudaMemcpyHostToDevice), "upload .440")) {
        if (a->d_data) cudaFree(a->d_data);
        a->d_data = nullptr;
        return ASSIST_ERROR_EPHEM_FILE;
    }
    return 0;
}

static void ascii_free(ascii_s* a) {
    if (!a) return;
    if (a->d_data) cudaFree(a->d_data);
    if (a->d_view) cudaFree(a->d_view);
    delete a;
}

static spk_s* spk_load(const char* path) {
    std::vector<unsigned char> b;
    if (!read_file(path, b) || b.size() < 1024) return nullptr;
    if (std::strncmp((const char*)b.data(), "DAF/SPK", 7) != 0) return nullptr;
    const int nd = get<int32_t>(b, 8), ni = get<int32_t>(b, 12);
    if (8 * (nd + (ni + 1) / 2) != 40) return nullptr;
    const int fward = get<int32_t>(b, 76);
    spk_s* s = new spk_s();
    long recno = fward;
    int guard = 0;
    while (recno > 0 && guard++ < 1000000) {
        const size_t ro = (size_t)(recno - 1) * 1024;
        if (ro + 1024 > b.size()) { delete s; return nullptr; }
        if (b[ro + 8] != 0 && s->targets.empty()) { delete s; return nullptr; }
        const double next = get<double>(b, ro), nsum = get<double>(b, ro + 16);
        if (!(nsum >= 0 && nsum <= 25)) { delete s; return nullptr; }
        for (int k = 0; k < (int)nsum; k++) {
            const size_t so = ro + 24 + 40 * (size_t)k;
            const double sbeg = get<double>(b, so), send = get<double>(b, so + 8);
            const int tar = get<int32_t>(b, so + 16), cen = get<int32_t>(b, so + 20);
            const int one = get<int32_t>(b, so + 32), two = get<int32_t>(b, so + 36);
            spk_target_h* t = nullptr;
            for (auto& x : s->targets) if (x.code == tar) { t = &x; break; }
            if (!t) {
                spk_target_h nt;
                nt.code = tar; nt.cen = cen; nt.mass = 0;
                nt.beg = 2451545.0 + sbeg / 86400.0;
                nt.res = (2451545.0 + send / 86400.0) - nt.beg;
                s->targets.push_back(nt);
                t = &s->targets.back();
            }
            t->one.push_back(one);
            t->two.push_back(two);
            t->end = 2451545.0 + send / 86400.0;
        }
        recno = (long)next;
    }
    s->data.resize(b.size() / 8);
    std::memcpy(s->data.data(), b.data(), s->data.size() * 8);
    /* comment records 2 .. fward-1: trailing NUL/EOT bytes of each record
     * dropped, NUL ends a line (src/spk.c:49-110) */
    for (int r = 0; r < fward - 2; r++) {
        const size_t o = (size_t)(1 + r) * 1024;
        if (o + 1024 > b.size()) break;
        int len = 1024;
        while (len > 0 && (b[o + len - 1] == 0 || b[o + len - 1] == 4)) len--;
        for (int k = 0; k < len; k++) s->comments.push_back(b[o + k] == 0 ? '\n' : (char)b[o + k]);
    }
    /* segment table with the per-call Julian-date conversions done once */
    for (auto& t : s->targets) {
        s->seg0.push_back((int)s->segs.size());
        for (size_t q = 0; q < t.one.size(); q++) {
            const long long two = t.two[q], one = t.one[q];
            if (two < 4 || (size_t)two > s->data.size() || one < 1 || one > two) { delete s; return nullptr; }
            const double* dir = s->data.data() + (two - 1);
            AgSpkSeg g;
            g.R = (int)dir[-1];
            g.P = (g.R - 2) / 3;
            g.nrec = (int)dir[0];
            if (g.R < 5 || g.P > AG_MAX_SPK_P || g.nrec < 1 || (long long)one - 1 + (long long)g.nrec * g.R > two) {
                delete s; return nullptr;
            }
            g.init_jd = 2451545.0 + dir[-3] / 86400.0;
            g.intlen_days = dir[-2] / 86400.0;
            g.inv_intlen_days = 1.0 / g.intlen_days;
            g.data_off = one - 1;
            g.meta_off = (int)s->meta.size();
            for (int r = 0; r < g.nrec; r++) {
                const double* val = s->data.data() + (one - 1) + (size_t)r * g.R;
                AgRecMeta m;
                m.x = 2451545.0 + val[0] / 86400.0;
                m.y = val[1] / 86400.0;
                m.z = 1.0 / m.y;
                m.w = 0.0;
                s->meta.push_back(m);
            }
            s->segs.push_back(g);
        }
    }
    return s;
}

/* The device copies of an SPK image, its segment table and record metadata,
 * made on first device use. */
static int spk_upload(spk_s* s) {
    if (s->d_data) return 0;
    bool ok = !ag_cuda_check(cudaMalloc(&s->d_data, s->data.size() * 8), "cudaMalloc(SPK)") &&
              !ag_cuda_check(cudaMemcpy(s->d_data, s->data.data(), s->data.size() * 8, cudaMemcpyHostToDevice), "upload SPK") &&
              !ag_cuda_check(cudaMalloc(&s->d_segs, sizeof(AgSpkSeg) * (s->segs.size() + 1)), "cudaMalloc(SPK segments)") &&
              !ag_cuda_check(cudaMemcpy(s->d_segs, s->segs.data(), sizeof(AgSpkSeg) * s->segs.size(), cudaMemcpyHostToDevice), "upload segments") &&
              !ag_cuda_check(cudaMalloc(&s->d_meta, sizeof(AgRecMeta) * (s->meta.size() + 1)), "cudaMalloc(SPK records)") &&
              !ag_cuda_check(cudaMemcpy(s->d_meta, s->meta.data(), sizeof(AgRecMeta) * s->meta.size(), cudaMemcpyHostToDevice), "upload records");
    if (!ok) {
        if (s->d_data) cudaFree(s->d_data);
        if (s->d_segs) cudaFree(s->d_segs);
        if (s->d_meta) cudaFree(s->d_meta);
        s->d_data = nullptr; s->d_segs = nullptr; s->d_meta = nullptr;
        return ASSIST_ERROR_EPHEM_FILE;
    }
    return 0;
}

static void spk_free(spk_s* s) {
    if (!s) return;
    if (s->d_data) cudaFree(s->d_data);
    if (s->d_segs) cudaFree(s->d_segs);
    if (s->d_meta) cudaFree(s->d_meta);
    if (s->d_view) cudaFree(s->d_view);
    delete s;
}

/* Constants and GMs of a planets SPK file: "KEY value" lines after "Initial
 * conditions and constants used for integration:", D exponents read as E
 * (src/spk.c:695-760). */
struct spk_constants {
    double AU = 0, EMRAT = 0, J2E = 0, J3E = 0, J4E = 0, J2SUN = 0, RE = 0, CLIGHT = 0, ASUN = 0;
    std::vector<std::pair<std::string, double>> masses;
};
static spk_constants spk_parse_constants(const std::string& c) {
    spk_constants k;
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
        const std::string K(key);
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

/* Masses of SPK targets by name (src/spk.c:137-200): planets from GMS,
 * GM1.., GMB (Earth and Moon split by EMRAT), asteroids from MAnnnn. */
static void spk_join_masses(spk_s* s, const spk_constants& k) {
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

/* ---------------------------------------------------------------- device view */
static void ag_ascii_view(const ascii_s* a, DevEphem& D);
static int ag_finish_view(const struct assist_ephem* e, DevEphem& D, DevEphem* out, bool may_upload = true);

/* The planets part of the view for a planets SPK file. */
static void spk_planets_view(const struct assist_ephem* e, DevEphem& D) {
    const spk_s* p = e->spk_planets;
    D.pl_spk = 1;
    D.pspk = p->d_data;
    D.psegs = p->d_segs;
    D.pmeta = p->d_meta;
    D.au_km = e->AU;
    D.pl_cau = e->AU;
    for (int k = 0; k <= ASSIST_BODY_NPLANETS; k++) {
        const int idx = k < ASSIST_BODY_NPLANETS ? e->spk_target_index[k] : e->spk_emb_index;
        D.ps_nseg[k] = 0;
        if (idx < 0) continue;
        const spk_target_h& t = p->targets[(size_t)idx];
        D.ps_seg0[k] = p->seg0[(size_t)idx];
        D.ps_nseg[k] = (int)t.one.size();
        D.ps_beg[k] = t.beg; D.ps_end[k] = t.end; D.ps_res[k] = t.res;
        if (k < ASSIST_BODY_NPLANETS) D.gm[k] = t.mass;
    }
}

int ag_ephem_device(const struct assist_ephem* e, DevEphem* out) {
    if (!e || (!e->ascii_planets && !e->spk_planets)) return ASSIST_ERROR_EPHEM_FILE;
    if ((e->spk_planets && spk_upload(e->spk_planets)) || (e->ascii_planets && ascii_upload(e->ascii_planets)) ||
        (e->spk_asteroids && spk_upload(e->spk_asteroids)))
        return ASSIST_ERROR_EPHEM_FILE;
    DevEphem D;
    std::memset(&D, 0, sizeof(D));
    D.jd_ref = e->jd_ref;
    if (e->spk_planets) spk_planets_view(e, D);
    else ag_ascii_view(e->ascii_planets, D);
    return ag_finish_view(e, D, out);
}

/* The planets part of the view for a .440/.441 file. */
static void ag_ascii_view(const ascii_s* a, DevEphem& D) {
    D.pl_data = a->d_data;
    D.pl_ndbl = (long long)a->data.size();
    D.pl_rec_len = (int)a->rec;
    D.pl_nrec = (int)(a->data.size() / a->rec);
    D.pl_beg = a->beg; D.pl_end = a->end; D.pl_inc = a->inc; D.pl_cau = a->cau; D.pl_cem = a->cem;
    for (int p = 0; p < 13; p++) {
        D.col_off[p] = a->off[p]; D.col_ncf[p] = a->ncf[p]; D.col_niv[p] = a->niv[p];
        D.col_vscale[p] = ((double)(a->niv[p] * 2) / a->inc / 86400.0) * (86400.0 / a->cau);
    }
    for (int k = 0; k < ASSIST_BODY_NPLANETS; k++) D.gm[k] = a->mass[k];
    D.inv_cau = 1.0 / a->cau;
    D.cau_per_day = a->cau / 86400.;
    D.f_earth = -1.0 / (1.0 + a->cem);
    D.f_moon = a->cem / (1.0 + a->cem);
    const double l2 = std::log2(a->inc);
    D.pl_inc_pow2 = (a->inc > 0 && std::floor(l2) == l2) ? 1 : 0;
    D.pl_inv_inc = 1.0 / a->inc;
}

/* Asteroids and constants, then the device copy of the view. */
static int ag_finish_view(const struct assist_ephem* e, DevEphem& D, DevEphem* out, bool may_upload) {
    const spk_s* s = e->spk_asteroids;
    D.n_ast = 0;
    if (s) {
        if ((int)s->targets.size() > AG_MAX_AST) return ASSIST_ERROR_NAST;
        D.n_ast = (int)s->targets.size();
        D.spk = s->d_data;
        D.spk_ndbl = (long long)s->data.size();
        D.segs = s->d_segs;
        D.rec_meta = s->d_meta;
        for (int m = 0; m < D.n_ast; m++) {
            const spk_target_h& t = s->targets[(size_t)m];
            D.ast_beg[m] = t.beg; D.ast_end[m] = t.end; D.ast_res[m] = t.res; D.ast_gm[m] = t.mass;
            D.ast_gm_hi[m] = (float)t.mass;
            D.ast_gm_lo[m] = (float)(t.mass - (double)D.ast_gm_hi[m]);
            D.ast_nseg[m] = (int)t.one.size();
            D.ast_seg0[m] = s->seg0[(size_t)m];
        }
    }
    D.J2E = e->J2E; D.J3E = e->J3E; D.J4E = e->J4E; D.J2SUN = e->J2SUN;
    D.Re_eq = e->Re_eq; D.Rs_eq = e->Rs_eq; D.c_squared = e->c_squared; D.over_c_squared = e->over_c_squared;
    /* the view is owned by the planets object (one view per ephemeris) */
    DevEphem** d_view = e->spk_planets ? &e->spk_planets->d_view : &e->ascii_planets->d_view;
    DevEphem* h_view = e->spk_planets ? &e->spk_planets->h_view : &e->ascii_planets->h_view;
    if (!may_upload) {
        /* the device view must exist and match the ephemeris as it is now */
        if (!*d_view) {
            ag_set_error("the ephemeris has no device view yet: make one ordinary device call with it first");
            return ASSIST_ERROR_EPHEM_FILE;
        }
        D.self_dev = *d_view;
        if (std::memcmp(h_view, &D, sizeof(D)) != 0) {
            ag_set_error("the ephemeris changed (jd_ref or a constant) since its device view was made: make one "
                         "ordinary device call with it first");
            return ASSIST_ERROR_EPHEM_FILE;
        }
        *out = D;
        return ASSIST_SUCCESS;
    }
    if (!*d_view && ag_cuda_check(cudaMalloc(d_view, sizeof(DevEphem)), "cudaMalloc(ephemeris view)"))
        return ASSIST_ERROR_EPHEM_FILE;
    D.self_dev = *d_view;
    if (std::memcmp(h_view, &D, sizeof(D)) != 0) {
        /* the view changed (first use, jd_ref or constants edited): refresh the device copy */
        if (ag_cuda_check(cudaMemcpy(*d_view, &D, sizeof(D), cudaMemcpyHostToDevice), "upload ephemeris view"))
            return ASSIST_ERROR_EPHEM_FILE;
        *h_view = D;
    }
    *out = D;
    return ASSIST_SUCCESS;
}

int ag_ephem_device_current(const struct assist_ephem* e, DevEphem* out) {
    if (!e || (!e->ascii_planets && !e->spk_planets)) return ASSIST_ERROR_EPHEM_FILE;
    if ((e->spk_planets && !e->spk_planets->d_data) || (e->ascii_planets && !e->ascii_planets->d_data) ||
        (e->spk_asteroids && !e->spk_asteroids->d_data)) {
        ag_set_error("the ephemeris has no device copy yet: make one ordinary device call with it first");
        return ASSIST_ERROR_EPHEM_FILE;
    }
    DevEphem D;
    std::memset(&D, 0, sizeof(D));
    D.jd_ref = e->jd_ref;
    if (e->spk_planets) spk_planets_view(e, D);
    else ag_ascii_view(e->ascii_planets, D);
    return ag_finish_view(e, D, out, false);
}

int ag_ephem_view_ready(const struct assist_ephem* e) {
    if (!e) return 0;
    if (e->spk_planets) return e->spk_planets->d_view ? 1 : 0;
    return e->ascii_planets && e->ascii_planets->d_view ? 1 : 0;
}

double ag_sun_gm(const struct assist_ephem* e) {
    if (e->spk_planets) {
        const int i = e->spk_target_index[ASSIST_BODY_SUN];
        return i >= 0 ? e->spk_planets->targets[(size_t)i].mass : 0.0;
    }
    return e->ascii_planets->mass[ASSIST_BODY_SUN];
}

int ag_ephem_n_bodies(const struct assist_ephem* e) {
    return ASSIST_BODY_NPLANETS + (e && e->spk_asteroids ? (int)e->spk_asteroids->targets.size() : 0);
}

/* Body evaluation through the device kernel (used by assist_all_ephem and
 * as ephem->planets_calc). */
extern "C" int ag_bodies_at(const struct assist_ephem* e, double t, double* out_all);

static enum ASSIST_STATUS ag_planets_calc(const struct assist_ephem* e, double jd_ref, double jd_rel, int body,
                                          double* const GM, double* const x, double* const y, double* const z,
                                          double* const vx, double* const vy, double* const vz, double* const ax,
                                          double* const ay, double* const az) {
    (void)jd_ref;
    if (body < 0 || body >= ASSIST_BODY_NPLANETS) return ASSIST_ERROR_NEPHEM;
    std::vector<double> all((size_t)ag_ephem_n_bodies(e) * 10);
    int st = ag_bodies_at(e, jd_rel, all.data());
    const double* o = all.data() + 10 * body;
    *GM = o[0]; *x = o[1]; *y = o[2]; *z = o[3]; *vx = o[4]; *vy = o[5]; *vz = o[6]; *ax = o[7]; *ay = o[8]; *az = o[9];
    if (st != ASSIST_SUCCESS) return (enum ASSIST_STATUS)st;
    return ASSIST_SUCCESS;
}

/* ---------------------------------------------------------------- front door */
extern "C" int assist_ephem_init(struct assist_ephem* ephem, char* user_planets_path, char* user_asteroids_path) {
    std::memset(ephem, 0, sizeof(*ephem));
    ephem->jd_ref = 2451545.0;
    for (int k = 0; k < ASSIST_BODY_NPLANETS; k++) ephem->spk_target_index[k] = -1;
    ephem->spk_emb_index = -1;
    const size_t FN = 1024;
    char planets[FN], asteroids[FN];
    const char* base = getenv("ASSIST_DIR");
    if (user_planets_path == nullptr && base == nullptr) return ASSIST_ERROR_EPHEM_FILE;
    if (user_planets_path == nullptr) {
        if (!assist_discover_planets_path(planets, FN, base)) std::snprintf(planets, FN, "%s%s", base, "/data/de441.bsp");
    } else {
        std::strncpy(planets, user_planets_path, FN - 1);
        planets[FN - 1] = '\0';
    }
    ephemeris_file_format_t fmt = FILE_FORMAT_UNKNOWN;
    int fd = open(planets, O_RDONLY);
    if (fd >= 0) { fmt = assist_detect_ephemeris_file_format(fd); close(fd); }
    bool ast_missing = false;
    if (user_asteroids_path == nullptr) {
        if (base == nullptr) ast_missing = true;
        else std::snprintf(asteroids, FN, "%s%s", base, "/data/sb441-n16.bsp");
    } else {
        std::strncpy(asteroids, user_asteroids_path, FN - 1);
        asteroids[FN - 1] = '\0';
    }
    if (!ast_missing) {
        ephem->spk_asteroids = spk_load(asteroids);
        if (!ephem->spk_asteroids) ast_missing = true;
    }
    if (fmt == FILE_FORMAT_ASCII_BIN) {
        ephem->ascii_planets = ascii_load(planets);
        if (!ephem->ascii_planets) {
            spk_free(ephem->spk_asteroids);
            ephem->spk_asteroids = nullptr;
            return ASSIST_ERROR_EPHEM_FILE;
        }
        const ascii_s* a = ephem->ascii_planets;
        ephem->planets_source = FILE_FORMAT_ASCII_BIN;
        ephem->J2E = a->J2E; ephem->J3E = a->J3E; ephem->J4E = a->J4E; ephem->J2SUN = a->J2SUN;
        ephem->AU = a->AU; ephem->RE = a->RE; ephem->CLIGHT = a->CLIGHT; ephem->ASUN = a->ASUN;
        ephem->EMRAT = a->cem;
        ephem->Re_eq = ephem->RE / ephem->AU;
        ephem->Rs_eq = ephem->ASUN / ephem->AU;
        ephem->c_AU_per_day = (ephem->CLIGHT / ephem->AU) * 86400.0;
        ephem->c_squared = ephem->c_AU_per_day * ephem->c_AU_per_day;
        ephem->over_c_squared = 1.0 / ephem->c_squared;
        ephem->planets_calc = ag_planets_calc;
        if (ephem->spk_asteroids) {
            for (auto& t : ephem->spk_asteroids->targets) {
                if (t.code >= 2000000) {
                    char key[16];
                    std::snprintf(key, sizeof(key), "MA%04d", t.code - 2000000);
                    double gm = 0.0;
                    if (a->find(key, &gm)) t.mass = gm;
                } else if (t.code == 399) t.mass = a->mass[ASSIST_BODY_EARTH];
                else if (t.code == 301) t.mass = a->mass[ASSIST_BODY_MOON];
                else if (t.code == 10) t.mass = a->mass[ASSIST_BODY_SUN];
            }
            if ((int)ephem->spk_asteroids->targets.size() > AG_MAX_AST) {
                std::fprintf(stderr, "(ASSIST) Asteroid file has more than %d targets.\n", AG_MAX_AST);
                spk_free(ephem->spk_asteroids);
                ephem->spk_asteroids = nullptr;
                ast_missing = true;
            }
        }
    } else if (fmt == FILE_FORMAT_VALID_BSP) {
        /* planets from an SPK file (src/assist.c:252-292) */
        spk_s* p = spk_load(planets);
        if (!p) {
            spk_free(ephem->spk_asteroids);
            ephem->spk_asteroids = nullptr;
            return ASSIST_ERROR_EPHEM_FILE;
        }
        ephem->spk_planets = p;
        ephem->planets_source = FILE_FORMAT_VALID_BSP;
        static const int naif_by_assist[ASSIST_BODY_NPLANETS] = {10, 1, 2, 399, 301, 4, 5, 6, 7, 8, 9};
        for (int k = 0; k < ASSIST_BODY_NPLANETS; k++)
            for (size_t i = 0; i < p->targets.size(); i++)
                if (p->targets[i].code == naif_by_assist[k]) { ephem->spk_target_index[k] = (int)i; break; }
        for (size_t i = 0; i < p->targets.size(); i++)
            if (p->targets[i].code == 3) { ephem->spk_emb_index = (int)i; break; }
        const spk_constants k = spk_parse_constants(p->comments);
        ephem->AU = k.AU; ephem->EMRAT = k.EMRAT; ephem->J2E = k.J2E; ephem->J3E = k.J3E; ephem->J4E = k.J4E;
        ephem->J2SUN = k.J2SUN; ephem->RE = k.RE; ephem->CLIGHT = k.CLIGHT; ephem->ASUN = k.ASUN;
        ephem->Re_eq = ephem->RE / ephem->AU;
        ephem->Rs_eq = ephem->ASUN / ephem->AU;
        ephem->c_AU_per_day = (ephem->CLIGHT / ephem->AU) * 86400;
        ephem->c_squared = ephem->c_AU_per_day * ephem->c_AU_per_day;
        ephem->over_c_squared = 1.0 / ephem->c_squared;
        spk_join_masses(p, k);
        spk_join_masses(ephem->spk_asteroids, k);
        ephem->planets_calc = ag_planets_calc;
        /* Earth and Moon are evaluated about the Earth-Moon barycentre */
        if (ephem->spk_emb_index < 0 || ephem->spk_target_index[ASSIST_BODY_EARTH] < 0 ||
            ephem->spk_target_index[ASSIST_BODY_MOON] < 0)
            std::fprintf(stderr, "(ASSIST) Planets SPK file lacks the Earth (399), Moon (301) or Earth-Moon barycentre (3).\n");
        if (ephem->spk_asteroids && (int)ephem->spk_asteroids->targets.size() > AG_MAX_AST) {
            std::fprintf(stderr, "(ASSIST) Asteroid file has more than %d targets.\n", AG_MAX_AST);
            spk_free(ephem->spk_asteroids);
            ephem->spk_asteroids = nullptr;
            ast_missing = true;
        }
    } else {
        spk_free(ephem->spk_asteroids);
        ephem->spk_asteroids = nullptr;
        std::fprintf(stderr, "(ASSIST) Error: Failed to initialize planets ephemeris from '%s'.\n", planets);
        return ASSIST_ERROR_EPHEM_FILE;
    }
    if (ast_missing) std::fprintf(stderr, "(ASSIST) %s\n", assist_error_messages[ASSIST_ERROR_AST_FILE]);
    return ASSIST_SUCCESS;
}

extern "C" void assist_ephem_free_pointers(struct assist_ephem* ephem) {
    if (!ephem) return;
    spk_free(ephem->spk_asteroids);
    spk_free(ephem->spk_planets);
    ascii_free(ephem->ascii_planets);
    ephem->spk_asteroids = nullptr;
    ephem->ascii_planets = nullptr;
    ephem->spk_planets = nullptr;
}

extern "C" void assist_ephem_free(struct assist_ephem* ephem) {
    if (!ephem) return;
    assist_ephem_free_pointers(ephem);
    std::free(ephem);
}

extern "C" struct assist_ephem* assist_ephem_create(char* planets, char* asteroids) {
    struct assist_ephem* e = (struct assist_ephem*)std::calloc(1, sizeof(struct assist_ephem));
    int err = assist_ephem_init(e, planets, asteroids);
    if (err != ASSIST_SUCCESS) {
        std::fprintf(stderr, "(ASSIST) An error occured while trying to initialize the ephemeris structure.\n");
        std::fprintf(stderr, "(ASSIST) %s\n", assist_error_messages[err]);
        assist_ephem_free(e);
        return nullptr;
    }
    return e;
}

extern "C" void assist_ephem_time_bounds(const struct assist_ephem* ephem, double* t_beg, double* t_end) {
    if (!ephem) return;
    double beg = -INFINITY, end = INFINITY;
    if (ephem->spk_planets) {
        for (auto& t : ephem->spk_planets->targets) {
            if (t.beg > beg) beg = t.beg;
            if (t.end < end) end = t.end;
        }
    } else if (ephem->ascii_planets) {
        if (ephem->ascii_planets->beg > beg) beg = ephem->ascii_planets->beg;
        if (ephem->ascii_planets->end < end) end = ephem->ascii_planets->end;
    }
    if (ephem->spk_asteroids)
        for (auto& t : ephem->spk_asteroids->targets) {
            if (t.beg > beg) beg = t.beg;
            if (t.end < end) end = t.end;
        }
    if (t_beg) *t_beg = beg - ephem->jd_ref;
    if (t_end) *t_end = end - ephem->jd_ref;
}
