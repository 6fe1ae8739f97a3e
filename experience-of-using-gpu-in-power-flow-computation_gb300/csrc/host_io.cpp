// host_io.cpp -- data.txt options, common-data-format reader/writer, grid
// construction and the seeded synthetic grid generator.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <numeric>
#include <queue>
#include <sstream>
#include <string>
#include <vector>

#include "gbpf_internal.h"

namespace gbpf {

static thread_local std::string g_last_error;
void set_error(const std::string &m) { g_last_error = m; }
const std::string &last_error() { return g_last_error; }

void Grid::rebuild_lists() {
    pv.clear();
    pq.clear();
    slack = 0;
    for (int k = 0; k < nB; k++) {
        if (type[k] == 0 || type[k] == 1) pq.push_back(k + 1);
        else if (type[k] == 2) pv.push_back(k + 1);
        else if (type[k] == 3) slack = k + 1;
    }
    nPV = (int)pv.size();
    nPQ = (int)pq.size();
}

}  // namespace gbpf

using gbpf::Grid;
using gbpf::set_error;

// ---------------------------------------------------------------------------
// data.txt: loadFile, GPU/sistInfo.h:62-242
// ---------------------------------------------------------------------------

namespace {

// Value lookup exactly as loadFile does it: the first occurrence of the key,
// then the first '=' at or after the end of the key (an absent key makes the
// std::string::npos arithmetic wrap, so the search starts near the beginning
// of the text), then `off` characters on, up to the next ';'.  The int
// conversions of the reference are kept (a missing '=' gives position 1).
bool lookup(const std::string &s, const std::string &key, int off, std::string *out) {
    size_t kp = s.find(key);
    size_t from = kp + key.size();  // wraps when kp == npos, as in the reference
    size_t eq = s.find('=', from);
    int inicio = (int)(uint32_t)(eq + (size_t)off);
    size_t fim = s.find(';', (size_t)(long long)inicio);
    size_t pos = (size_t)(long long)inicio;
    if (pos > s.size()) return false;  // std::string::substr would throw
    *out = s.substr(pos, fim - pos);
    return true;
}

struct Echo {
    std::string text;
    void line(const std::string &l) { text += l; text += '\n'; }
};

std::string fmt_g(double v) {  // std::cout << double with default flags
    char b[64];
    std::snprintf(b, sizeof b, "%g", v);
    return b;
}
std::string fmt_f(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%f", v);
    return b;
}

}  // namespace

extern "C" gbpf_status gbpf_options_default(gbpf_options *o) {
    if (!o) return GBPF_E_ARG;
    std::memset(o, 0, sizeof *o);
    o->metodo = GBPF_METODO_NDA;  // global::metodo is value-initialised then set by loadFile
    o->v_inicial = 1.0;
    o->theta_inicial = 0.0;
    o->tolerancia = 0.0001;
    o->no_max_iter = 100;
    o->lim_inj_reat = 0;
    o->openmp = 1;
    o->laconic_mode = 0;
    o->verbose_mode = 0;
    o->output_ans = 1;
    o->output_iter = 0;
    o->streams = 1;
    o->output_bench = GBPF_BENCH_ALL;
    o->precision = GBPF_PREC_FP64;
    std::snprintf(o->arq_entrada, sizeof o->arq_entrada, "%s", "ieee14.cdf");
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_options_parse(const char *text, gbpf_options *o, char *echo,
                                          size_t echo_cap) {
    if (!text || !o) return GBPF_E_ARG;
    const std::string str(text);
    Echo E;
    std::string aux;
    auto need = [&](const char *key, int off) -> bool {
        if (!lookup(str, key, off, &aux)) {
            set_error(std::string("data.txt: value of '") + key + "' starts past the end of the text");
            return false;
        }
        return true;
    };
    if (!need("laconic_mode", 2)) return GBPF_E_INPUT;
    const std::string laconic_aux = aux;
    o->laconic_mode = (aux == "OFF") ? 0 : 1;
    const bool loud = !o->laconic_mode;

    if (!need("metodo", 2)) return GBPF_E_INPUT;
    if (loud) E.line("metodo         = " + aux);
    if (aux == "denso") o->metodo = GBPF_METODO_DENSO;
    else if (aux == "esparso") o->metodo = GBPF_METODO_ESPARSO;
    else if (aux == "hibridoA") o->metodo = GBPF_METODO_HIBRIDOA;
    else if (aux == "hibridoB") o->metodo = GBPF_METODO_HIBRIDOB;
    else if (aux == "hibridoC") o->metodo = GBPF_METODO_HIBRIDOC;
    else o->metodo = GBPF_METODO_NDA;

    if (!need("lim_inj_reat", 2)) return GBPF_E_INPUT;
    if (loud && str.find("lim_inj_reat") != std::string::npos) E.line("lim_inj_reat   = " + aux);
    if (aux == "OFF") o->lim_inj_reat = 0;
    else if (aux == "ON") o->lim_inj_reat = 1;

    if (!need("openmp", 2)) return GBPF_E_INPUT;
    if (loud) E.line("openmp         = " + aux);
    o->openmp = (aux == "OFF") ? 0 : 1;

    if (!need("v_inicial", 1)) return GBPF_E_INPUT;
    o->v_inicial = std::atof(aux.c_str());
    if (loud) E.line("v_inicial      = " + fmt_f(o->v_inicial));

    if (!need("theta_inicial", 1)) return GBPF_E_INPUT;
    o->theta_inicial = std::atof(aux.c_str());
    if (loud) E.line("theta_inicial  = " + fmt_f(o->theta_inicial));

    if (!need("tolerancia", 1)) return GBPF_E_INPUT;
    o->tolerancia = std::atof(aux.c_str());
    if (loud) E.line("tolerancia     = " + fmt_g(o->tolerancia));

    if (!need("no_max_iter", 1)) return GBPF_E_INPUT;
    {
        // std::stoi: leading blanks, optional sign, at least one digit
        const char *p = aux.c_str();
        while (std::isspace((unsigned char)*p)) p++;
        const char *q = p;
        if (*q == '+' || *q == '-') q++;
        if (!std::isdigit((unsigned char)*q)) {
            set_error("data.txt: no_max_iter is not an integer");
            return GBPF_E_INPUT;
        }
        o->no_max_iter = std::atoi(p);
    }
    if (loud) E.line("no_max_iter    = " + std::to_string(o->no_max_iter));

    if (!need("arq_entrada", 2)) return GBPF_E_INPUT;
    std::snprintf(o->arq_entrada, sizeof o->arq_entrada, "%s", aux.c_str());
    if (loud) E.line("arq_entrada    = " + aux);

    if (!need("verbose_mode", 2)) return GBPF_E_INPUT;
    if (loud && str.find("verbose_mode") != std::string::npos) E.line("verbose_mode   = " + aux);
    if (aux == "OFF") o->verbose_mode = 0;
    else if (aux == "ON") o->verbose_mode = 1;

    if (loud) E.line("laconic_mode   = " + laconic_aux);

    if (!need("output_bench", 2)) return GBPF_E_INPUT;
    if (loud) E.line("output_bench   = " + aux);
    if (aux == "ALL") o->output_bench = GBPF_BENCH_ALL;
    else if (aux == "FILE") o->output_bench = GBPF_BENCH_FILE;
    else o->output_bench = GBPF_BENCH_SCREEN;

    if (!need("output_ans", 2)) return GBPF_E_INPUT;
    if (loud) E.line("output_ans     = " + aux);
    o->output_ans = (aux == "OFF") ? 0 : 1;

    if (!need("output_iter", 2)) return GBPF_E_INPUT;
    if (loud && str.find("output_iter") != std::string::npos) E.line("output_iter    = " + aux);
    if (aux == "OFF") o->output_iter = 0;
    else if (aux == "ON") o->output_iter = 1;

    if (!need("streams", 2)) return GBPF_E_INPUT;
    if (loud && str.find("streams") != std::string::npos) E.line("streams        = " + aux);
    if (aux == "OFF") o->streams = 0;
    else if (aux == "ON") o->streams = 1;

    // Keys this engine adds; the reference ignores them.  Only read when present.
    if (str.find("precisao") != std::string::npos && lookup(str, "precisao", 2, &aux)) {
        if (aux == "FP32") o->precision = GBPF_PREC_FP32_IR;
        else if (aux == "FP64") o->precision = GBPF_PREC_FP64;
    }
    if (echo && echo_cap) std::snprintf(echo, echo_cap, "%s", E.text.c_str());
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_options_load(const char *path, gbpf_options *o, char *echo,
                                         size_t echo_cap) {
    if (!path || !o) return GBPF_E_ARG;
    std::ifstream t(path, std::ios::binary);
    if (!t) {
        set_error(std::string("cannot open ") + path);
        return GBPF_E_INPUT;
    }
    std::ostringstream ss;
    ss << t.rdbuf();
    return gbpf_options_parse(ss.str().c_str(), o, echo, echo_cap);
}

// ---------------------------------------------------------------------------
// Common data format reader: GPU/sistema.h:386-638 (.cdf), GPU/arquivo.h:4-248 (.cdfx)
// ---------------------------------------------------------------------------

namespace {

struct Cols {
    int id_p, id_l, type_p, v_p, th_p, pl_p, ql_p, pg_p, qg_p, vb_p, qmax_p, qmin_p, gsh_p, bsh_p;
    int de_p, de_l, pa_p, r_p, x_p, b_p, tap_p, phi_p;
};
// Column starts of GPU/sistema.h:486-593 and GPU/arquivo.h:96-203 (widths are
// fixed by the substr calls and live in the readers below).
const Cols CDF_COLS = {0, 4, 24, 27, 33, 40, 49, 59, 67, 76, 90, 98, 106, 114,
                       0, 4, 4, 19, 29, 40, 76, 83};
const Cols CDFX_COLS = {0, 5, 25, 28, 34, 41, 50, 60, 68, 77, 91, 99, 107, 115,
                        0, 5, 6, 21, 31, 42, 78, 85};

constexpr double PI_REF = 3.14159265358979323846;  // GPU/sistema.h:526

struct Field {
    bool bad = false;
    std::string sub(const std::string &l, size_t pos, size_t len) {
        if (pos > l.size()) { bad = true; return std::string(); }
        return l.substr(pos, len);
    }
    int i(const std::string &l, size_t pos, size_t len) { return std::atoi(sub(l, pos, len).c_str()); }
    double d(const std::string &l, size_t pos, size_t len) { return std::atof(sub(l, pos, len).c_str()); }
};

// Smith's (1962) complex division, used for the parallel-branch merge.
void cdiv(double a, double b, double c, double d, double *re, double *im) {
    if (std::fabs(c) >= std::fabs(d)) {
        double r = d / c, den = c + d * r;
        *re = (a + b * r) / den;
        *im = (b - a * r) / den;
    } else {
        double r = c / d, den = c * r + d;
        *re = (a * r + b) / den;
        *im = (b * r - a) / den;
    }
}

// ---------------------------------------------------------------------------
// MATPOWER case reader: lerArquivoMatPOWEReficiente (GPU/m.h:485-599) with
// cleanLine / readMatrix (GPU/m.h:445-483) and storeMatPOWER (GPU/m.h:296-443).
// A grid read here takes calcYbusSp_Matpower's branch stamps (GPU/main.cu:78-81).
// ---------------------------------------------------------------------------

// cleanLine: drop a '%' comment, then trailing blanks, one ';' and blanks
// ('\r' counts as a blank, so CRLF files read like LF files).
void m_clean(std::string &s) {
    const size_t c = s.find('%');
    if (c != std::string::npos) s.resize(c);
    auto blank = [](char ch) { return ch == ' ' || ch == '\t' || ch == '\r'; };
    while (!s.empty() && blank(s.back())) s.pop_back();
    if (!s.empty() && s.back() == ';') s.pop_back();
    while (!s.empty() && blank(s.back())) s.pop_back();
}

// Removes the first "mpc.<name>[ \t]*=[ \t]*" (and '[' when `bracket`) from s,
// as the regex_search / regex_replace pairs of GPU/m.h:505-536 do.
bool m_take(std::string &s, const std::string &name, bool bracket) {
    const std::string key = "mpc." + name;
    for (size_t p = s.find(key); p != std::string::npos; p = s.find(key, p + 1)) {
        size_t q = p + key.size();
        while (q < s.size() && (s[q] == ' ' || s[q] == '\t')) q++;
        if (q >= s.size() || s[q] != '=') continue;
        q++;
        while (q < s.size() && (s[q] == ' ' || s[q] == '\t')) q++;
        if (bracket) {
            if (q >= s.size() || s[q] != '[') continue;
            q++;
        }
        s.erase(p, q - p);
        return true;
    }
    return false;
}

// One matrix row: tokens split on tabs (the reference's tokenize(line, "\t"),
// GPU/m.h:122-142) or blanks, each read by strtod like std::stod.  False when
// a token does not start with a number (std::stod would throw there).
bool m_row(const std::string &s, std::vector<std::vector<double>> &rows) {
    std::vector<double> r;
    const char *p = s.c_str();
    for (;;) {
        while (*p == '\t' || *p == ' ' || *p == '\r') p++;
        if (!*p) break;
        char *end;
        const double v = std::strtod(p, &end);
        if (end == p) return false;
        while (*end && *end != '\t' && *end != ' ' && *end != '\r') end++;
        r.push_back(v);
        p = end;
    }
    if (!r.empty()) rows.push_back(std::move(r));
    return true;
}

gbpf_status read_m(const std::string &path, double v0, double th0, Grid &g, std::string &err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "Erro na leitura do arquivo. Ele existe? " + path; return GBPF_E_INPUT; }
    static const char *NAMES[3] = {"bus", "gen", "branch"};
    std::vector<std::vector<double>> M[3];
    double base = 0;
    bool have_base = false, bad = false;
    std::string line;
    while (std::getline(f, line)) {
        m_clean(line);
        if (line.empty()) continue;
        for (int k = 0; k < 3; k++) {
            if (!m_take(line, NAMES[k], true)) continue;
            // readMatrix: rows up to and including the line that holds ']'
            for (;;) {
                const bool last = line.find(']') != std::string::npos;
                if (last) line.erase(std::remove(line.begin(), line.end(), ']'), line.end());
                m_clean(line);
                if (!line.empty() && !m_row(line, M[k])) bad = true;
                if (last || !std::getline(f, line)) break;
            }
            break;
        }
        if (m_take(line, "baseMVA", false)) {
            line.erase(std::remove_if(line.begin(), line.end(), [](char c) { return c == '"' || c == '\''; }),
                       line.end());
            char *end;
            base = std::strtod(line.c_str(), &end);
            have_base = end != line.c_str();
        }
    }
    if (bad) { err = "a matrix entry of the .m file is not a number"; return GBPF_E_INPUT; }
    if (!have_base) { err = "mpc.baseMVA not found"; return GBPF_E_INPUT; }
    // columns this reader uses: bus BUS_I..BASE_KV, gen GEN_BUS..QMIN, branch F_BUS..SHIFT
    static const size_t NEED[3] = {10, 5, 10};
    for (int k = 0; k < 3; k++)
        for (size_t i = 0; i < M[k].size(); i++)
            if (M[k][i].size() < NEED[k]) {
                err = std::string("mpc.") + NAMES[k] + " row " + std::to_string(i + 1) + " has " +
                      std::to_string(M[k][i].size()) + " columns, " + std::to_string(NEED[k]) + " needed";
                return GBPF_E_INPUT;
            }
    const auto &B = M[0], &G = M[1], &R = M[2];
    int nsl = 0;
    for (const auto &b : B) {
        const int t = (int)b[1];
        if (t < 1 || t > 3) { err = "ERRO: valor de tipo de barra invalido! (" + std::to_string(t) + ")"; return GBPF_E_INPUT; }
        nsl += t == 3;
    }
    if (nsl != 1) {
        err = nsl ? "ERRO: mais de uma barrra swing definida!" : "no slack bus (type 3) in the file";
        return GBPF_E_INPUT;
    }
    const int nB = (int)B.size();
    g = Grid();
    g.nB = nB;
    g.baseMVA = base;
    g.ybus_form = GBPF_YBUS_MATPOWER;
    g.id.assign(nB, 0); g.type.assign(nB, 0);
    g.V0.assign(nB, v0); g.theta0.assign(nB, th0);
    g.Pload.assign(nB, 0); g.Qload.assign(nB, 0); g.Pg.assign(nB, 0); g.Qg.assign(nB, 0);
    g.gsh.assign(nB, 0); g.bsh.assign(nB, 0); g.Vbase.assign(nB, 0);
    std::vector<double> qmax_bus(nB, 0), qmin_bus(nB, 0);
    for (int k = 0; k < nB; k++) {
        const auto &b = B[k];
        const int t = (int)b[1];
        g.id[k] = (int)b[0];
        g.type[k] = t == 1 ? 0 : t;  // MATPOWER PQ = 1 is the CDF's 0
        int gi = -1;
        if (t != 1) {
            // the first generator row on the bus (std::find over GEN_BUS); a
            // generator on a PQ bus is never looked up
            for (size_t j = 0; j < G.size(); j++)
                if ((int)G[j][0] == g.id[k]) { gi = (int)j; break; }
            g.V0[k] = b[7];
            if (t == 3) g.theta0[k] = b[8] * PI_REF / 180.;
            if (gi < 0) {
                g.notices.push_back("barra " + std::to_string(g.id[k]) + ", de tipo " + (t == 2 ? "PV" : "VO") +
                                    ", n\xc3\xa3o possui de gera\xc3\xa7\xc3\xa3o!");
            } else if (t == 2) {
                qmax_bus[k] = G[gi][3] / base;
                qmin_bus[k] = G[gi][4] / base;
            }
        }
        g.Pload[k] = b[2] / base;
        g.Qload[k] = b[3] / base;
        g.Pg[k] = gi < 0 ? 0 : G[gi][1] / base;
        g.Qg[k] = gi < 0 ? 0 : G[gi][2] / base;
        g.Vbase[k] = b[9];
        g.bsh[k] = b[5] / base;
        g.gsh[k] = b[4] / base;
    }
    g.rebuild_lists();
    for (int i = 0; i < g.nPV; i++) {
        const int k = g.pv[i] - 1;
        g.Qmax.push_back(qmax_bus[k]);
        g.Qmin.push_back(qmin_bus[k]);
        g.Vset.push_back(g.V0[k]);
    }
    // branches: id2i (GPU/sistema.h:465-472), every row its own branch (the
    // reference's storeMatPOWER never merges repeated pairs)
    for (const auto &r : R) {
        const int idde = (int)r[0], idpa = (int)r[1];
        int de = 0, pa = 0;
        for (int b = 0; b < nB; b++) if (g.id[b] == idde) { de = b + 1; break; }
        for (int b = 0; b < nB; b++) if (g.id[b] == idpa) { pa = b + 1; break; }
        if (!de || !pa) {
            err = "branch " + std::to_string(idde) + "-" + std::to_string(idpa) + " names an unknown bus";
            return GBPF_E_INPUT;
        }
        const double a = r[8], ph = r[9] * PI_REF / 180.;
        g.de.push_back(de); g.para.push_back(pa);
        g.r.push_back(r[2]); g.x.push_back(r[3]); g.bch.push_back(r[4]);
        g.phase.push_back(ph);
        if (a != 0.) { g.tap_re.push_back(a * std::cos(ph)); g.tap_im.push_back(a * std::sin(ph)); }
        else { g.tap_re.push_back(std::cos(ph)); g.tap_im.push_back(std::sin(ph)); }
        g.nL++;
    }
    return GBPF_OK;
}

gbpf_status read_cdf(const std::string &path, double v0, double th0, Grid &g, std::string &err) {
    const size_t dot = path.find_last_of('.');
    std::string ext = dot == std::string::npos ? std::string() : path.substr(dot + 1);
    std::transform(ext.begin(), ext.end(), ext.begin(), ::tolower);
    const Cols *C;
    if (ext == "cdf") C = &CDF_COLS;
    else if (ext == "cdfx") C = &CDFX_COLS;
    else if (ext == "m") return read_m(path, v0, th0, g, err);
    else { err = "nda == " + ext; return GBPF_E_INPUT; }

    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "ERRO: arquivo .cdf nao pode ser aberto: " + path; return GBPF_E_INPUT; }
    std::vector<std::string> L;
    std::string line;
    while (std::getline(f, line)) L.push_back(line);
    if (L.size() < 2) { err = "truncated file"; return GBPF_E_INPUT; }
    Field F;
    // lerTamanhos: bus lines until a line containing "-999"
    size_t li = 2;
    int nslack = 0, nB = 0;
    for (; li < L.size(); li++) {
        if (L[li].find("-999") != std::string::npos) break;
        int t = F.i(L[li], C->type_p, 2);
        if (t < 0 || t > 3) { err = "ERRO: valor de tipo de barra invalido!"; return GBPF_E_INPUT; }
        if (t == 3) nslack++;
        nB++;
    }
    if (nslack != 1) {
        err = nslack ? "ERRO: mais de uma barrra swing definida!" : "no slack bus (type 3) in the file";
        return GBPF_E_INPUT;
    }
    const size_t bus0 = 2, br0 = li + 2;
    g = Grid();
    g.nB = nB;
    g.baseMVA = (double)F.i(L[0], 31, 6);
    const double base = g.baseMVA;
    g.id.assign(nB, 0); g.type.assign(nB, 0);
    g.V0.assign(nB, v0); g.theta0.assign(nB, th0);
    g.Pload.assign(nB, 0); g.Qload.assign(nB, 0); g.Pg.assign(nB, 0); g.Qg.assign(nB, 0);
    g.gsh.assign(nB, 0); g.bsh.assign(nB, 0); g.Vbase.assign(nB, 0);
    std::vector<double> qmax_bus(nB, 0), qmin_bus(nB, 0);
    for (int k = 0; k < nB; k++) {
        const std::string &s = L[bus0 + k];
        g.id[k] = F.i(s, C->id_p, C->id_l);
        const int t = F.i(s, C->type_p, 2);
        g.type[k] = t;
        if (t == 2) {
            g.V0[k] = F.d(s, C->v_p, 6);
            qmax_bus[k] = F.d(s, C->qmax_p, 7) / base;
            qmin_bus[k] = F.d(s, C->qmin_p, 7) / base;
        } else if (t == 3) {
            g.V0[k] = F.d(s, C->v_p, 6);
            g.theta0[k] = F.d(s, C->th_p, 7) * PI_REF / 180.;
        }
        g.Pload[k] = F.d(s, C->pl_p, 9) / base;
        g.Qload[k] = F.d(s, C->ql_p, 10) / base;
        g.Pg[k] = F.d(s, C->pg_p, 8) / base;
        g.Qg[k] = F.d(s, C->qg_p, 8) / base;
        g.Vbase[k] = F.d(s, C->vb_p, 7);
        g.bsh[k] = F.d(s, C->bsh_p, 8);
        g.gsh[k] = F.d(s, C->gsh_p, 8);
    }
    g.rebuild_lists();
    for (int i = 0; i < g.nPV; i++) {
        const int k = g.pv[i] - 1;
        g.Qmax.push_back(qmax_bus[k]);
        g.Qmin.push_back(qmin_bus[k]);
        g.Vset.push_back(g.V0[k]);
    }
    // branches: id2i (GPU/sistema.h:465-472) and the merge of a repeated
    // (de, para) pair into a parallel equivalent (GPU/sistema.h:595-625)
    std::vector<int> idmap_keys(g.id);
    for (size_t bl = br0; bl < L.size(); bl++) {
        const std::string &s = L[bl];
        if (s.find("-999") != std::string::npos) break;
        const int idde = F.i(s, C->de_p, C->de_l), idpa = F.i(s, C->pa_p, 5);
        int de = 0, pa = 0;
        for (int b = 0; b < nB; b++) if (g.id[b] == idde) { de = b + 1; break; }
        for (int b = 0; b < nB; b++) if (g.id[b] == idpa) { pa = b + 1; break; }
        if (!de || !pa) {
            err = "branch " + std::to_string(idde) + "-" + std::to_string(idpa) + " names an unknown bus";
            return GBPF_E_INPUT;
        }
        const double r = F.d(s, C->r_p, 10), x = F.d(s, C->x_p, 11), bch = F.d(s, C->b_p, 10);
        const double a = F.d(s, C->tap_p, 6), ph = F.d(s, C->phi_p, 7) * PI_REF / 180.;
        double tre, tim;
        if (a != 0.) { tre = a * std::cos(ph); tim = a * std::sin(ph); }
        else { tre = std::cos(ph); tim = std::sin(ph); }
        int dup = -1;
        for (int b = 0; b < g.nL; b++) if (g.de[b] == de && g.para[b] == pa) { dup = b; break; }
        if (dup < 0) {
            g.de.push_back(de); g.para.push_back(pa);
            g.r.push_back(r); g.x.push_back(x); g.bch.push_back(bch);
            g.tap_re.push_back(tre); g.tap_im.push_back(tim); g.phase.push_back(ph);
            g.nL++;
        } else {
            // the two notices of GPU/sistema.h:596-611; the first names the most
            // recently added branch, as the reference's printf does
            char b[256];
            std::snprintf(b, sizeof b, "Ramo %d-%d declarado duas vezes. Criando equivalente paralelo...",
                          g.de[g.nL - 1], g.para[g.nL - 1]);
            g.notices.push_back(b);
            if (tre != g.tap_re[dup] || tim != g.tap_im[dup]) {
                std::snprintf(b, sizeof b, "Atencao! Os parametros lidos para os transformadores de potencia "
                              "das linhas de transmiss\xc3\xa3o paralelas s\xc3\xa3o diferentes! (linha %d)", dup);
                g.notices.push_back(b);
            }
            const double nr = r * g.r[dup] - x * g.x[dup], ni = r * g.x[dup] + x * g.r[dup];
            cdiv(nr, ni, g.r[dup] + r, g.x[dup] + x, &g.r[dup], &g.x[dup]);
            // the reference's merge rule for the charging, kept as is (GPU/sistema.h:620-624)
            if (bch != 0 || g.bch[dup] != 0) g.bch[dup] = 1 / (bch + g.bch[dup]);
            else g.bch[dup] = 0;
        }
    }
    if (F.bad) { err = "a fixed-width field starts past the end of its line"; return GBPF_E_INPUT; }
    return GBPF_OK;
}

}  // namespace

extern "C" gbpf_status gbpf_grid_read(const char *path, double v_inicial, double theta_inicial,
                                      gbpf_grid **out, char *msg, size_t msg_cap) {
    if (!path || !out) return GBPF_E_ARG;
    *out = nullptr;
    auto *h = new gbpf_grid;
    std::string err;
    gbpf_status st = read_cdf(path, v_inicial, theta_inicial, h->g, err);
    if (st != GBPF_OK) {
        set_error(err);
        if (msg && msg_cap) std::snprintf(msg, msg_cap, "%s", err.c_str());
        delete h;
        return st;
    }
    if (msg && msg_cap) {
        std::string all;
        for (auto &n : h->g.notices) { all += n; all += '\n'; }
        std::snprintf(msg, msg_cap, "%s", all.c_str());
    }
    *out = h;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_grid_create(const gbpf_grid_desc *d, gbpf_grid **out) {
    if (!d || !out || d->nB <= 1 || d->nL < 0 || !d->bus_type || !d->V0 || !d->theta0 ||
        (d->nL && (!d->from_bus || !d->to_bus || !d->r || !d->x)))
        return GBPF_E_ARG;
    *out = nullptr;
    auto *h = new gbpf_grid;
    Grid &g = h->g;
    const int n = d->nB;
    g.nB = n;
    g.baseMVA = d->baseMVA > 0 ? d->baseMVA : 100.0;
    auto cp = [n](const double *p, double dflt) {
        std::vector<double> v(n, dflt);
        if (p) std::copy(p, p + n, v.begin());
        return v;
    };
    g.type.assign(d->bus_type, d->bus_type + n);
    g.id.resize(n);
    for (int k = 0; k < n; k++) g.id[k] = d->id ? d->id[k] : k + 1;
    g.V0 = cp(d->V0, 1.0); g.theta0 = cp(d->theta0, 0.0);
    g.Pload = cp(d->Pload, 0); g.Qload = cp(d->Qload, 0); g.Pg = cp(d->Pg, 0); g.Qg = cp(d->Qg, 0);
    g.gsh = cp(d->gsh, 0); g.bsh = cp(d->bsh, 0); g.Vbase.assign(n, 0);
    int ns = 0;
    for (int k = 0; k < n; k++) {
        if (g.type[k] < 0 || g.type[k] > 3) { delete h; set_error("bus_type must be 0..3"); return GBPF_E_INPUT; }
        ns += g.type[k] == 3;
    }
    if (ns != 1) { delete h; set_error("exactly one slack bus (type 3) is required"); return GBPF_E_INPUT; }
    g.rebuild_lists();
    for (int i = 0; i < g.nPV; i++) {
        const int k = g.pv[i] - 1;
        g.Qmax.push_back(d->Qmax ? d->Qmax[k] : 0.0);
        g.Qmin.push_back(d->Qmin ? d->Qmin[k] : 0.0);
        g.Vset.push_back(g.V0[k]);
    }
    g.nL = d->nL;
    for (int b = 0; b < d->nL; b++) {
        const int f = d->from_bus[b], t = d->to_bus[b];
        if (f < 1 || f > n || t < 1 || t > n || f == t) {
            delete h;
            set_error("branch " + std::to_string(b) + " has an invalid bus index");
            return GBPF_E_INPUT;
        }
        g.de.push_back(f); g.para.push_back(t);
        g.r.push_back(d->r[b]); g.x.push_back(d->x[b]);
        g.bch.push_back(d->bch ? d->bch[b] : 0.0);
        g.tap_re.push_back(d->tap_re ? d->tap_re[b] : 1.0);
        g.tap_im.push_back(d->tap_im ? d->tap_im[b] : 0.0);
        g.phase.push_back(d->phase ? d->phase[b] : 0.0);
    }
    *out = h;
    return GBPF_OK;
}

extern "C" void gbpf_grid_free(gbpf_grid *g) { delete g; }

extern "C" gbpf_status gbpf_grid_dims(const gbpf_grid *h, int dims[8]) {
    if (!h || !dims) return GBPF_E_ARG;
    const Grid &g = h->g;
    gbpf::YPattern y = gbpf::build_ypattern(g);
    dims[0] = g.nB; dims[1] = g.nL; dims[2] = g.nPV; dims[3] = g.nPQ; dims[4] = g.slack;
    dims[5] = y.nnz; dims[6] = (int)g.baseMVA; dims[7] = (int)g.notices.size();
    return GBPF_OK;
}

template <class T>
static void put(T *dst, const std::vector<T> &src) {
    if (dst && !src.empty()) std::copy(src.begin(), src.end(), dst);
}

extern "C" gbpf_status gbpf_grid_buses(const gbpf_grid *h, int *id, int *type, double *V0,
                                       double *theta0, double *Pload, double *Qload, double *Pg,
                                       double *Qg, double *gsh, double *bsh) {
    if (!h) return GBPF_E_ARG;
    const Grid &g = h->g;
    put(id, g.id); put(type, g.type); put(V0, g.V0); put(theta0, g.theta0);
    put(Pload, g.Pload); put(Qload, g.Qload); put(Pg, g.Pg); put(Qg, g.Qg);
    put(gsh, g.gsh); put(bsh, g.bsh);
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_grid_pvpq(const gbpf_grid *h, int *pv, double *Qmin, double *Qmax,
                                      double *Vset, int *pq) {
    if (!h) return GBPF_E_ARG;
    const Grid &g = h->g;
    put(pv, g.pv); put(Qmin, g.Qmin); put(Qmax, g.Qmax); put(Vset, g.Vset); put(pq, g.pq);
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_grid_branches(const gbpf_grid *h, int *from_bus, int *to_bus,
                                          double *r, double *x, double *bch, double *tap_re,
                                          double *tap_im, double *phase) {
    if (!h) return GBPF_E_ARG;
    const Grid &g = h->g;
    put(from_bus, g.de); put(to_bus, g.para); put(r, g.r); put(x, g.x); put(bch, g.bch);
    put(tap_re, g.tap_re); put(tap_im, g.tap_im); put(phase, g.phase);
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_grid_set_buses(gbpf_grid *h, const double *Pload, const double *Qload,
                                           const double *Pg, const double *Qg, const double *V0,
                                           const double *theta0) {
    if (!h) return GBPF_E_ARG;
    Grid &g = h->g;
    const int n = g.nB;
    if (Pload) std::copy(Pload, Pload + n, g.Pload.begin());
    if (Qload) std::copy(Qload, Qload + n, g.Qload.begin());
    if (Pg) std::copy(Pg, Pg + n, g.Pg.begin());
    if (Qg) std::copy(Qg, Qg + n, g.Qg.begin());
    if (V0) {
        std::copy(V0, V0 + n, g.V0.begin());
        for (int i = 0; i < g.nPV; i++) g.Vset[i] = g.V0[g.pv[i] - 1];
    }
    if (theta0) std::copy(theta0, theta0 + n, g.theta0.begin());
    return GBPF_OK;
}

// ---------------------------------------------------------------------------
// CDF writer (fixed columns read back by the reader above)
// ---------------------------------------------------------------------------

extern "C" gbpf_status gbpf_grid_write_cdf(const gbpf_grid *h, const char *path, const char *title) {
    if (!h || !path) return GBPF_E_ARG;
    const Grid &g = h->g;
    const bool wide = g.nB > 9999;  // 4-digit ids do not fit: write the CDFX layout
    std::string p(path);
    FILE *f = std::fopen(path, "wb");
    if (!f) { set_error(std::string("cannot write ") + path); return GBPF_E_INPUT; }
    const int sh = wide ? 1 : 0;
    auto pad = [](std::string &s, size_t col) { if (s.size() < col) s.append(col - s.size(), ' '); };
    auto putf = [&](std::string &s, size_t col, const char *fmtstr, double v, size_t width) {
        pad(s, col);
        char b[64];
        std::snprintf(b, sizeof b, fmtstr, v);
        std::string t(b);
        if (t.size() > width) t = t.substr(0, width);
        if (t.size() < width) t = std::string(width - t.size(), ' ') + t;
        s.resize(col);
        s += t;
    };
    char hdr[128];
    std::snprintf(hdr, sizeof hdr, " 12/03/26 GBPF SYNTHETIC        %5.1f  2026 W %s", g.baseMVA,
                  title ? title : "synthetic grid");
    std::fprintf(f, "%s\r\n", hdr);
    std::fprintf(f, "BUS DATA FOLLOWS                          %5d ITEMS\r\n", g.nB);
    std::vector<double> qmax(g.nB, 0), qmin(g.nB, 0);
    for (int i = 0; i < g.nPV; i++) { qmax[g.pv[i] - 1] = g.Qmax[i]; qmin[g.pv[i] - 1] = g.Qmin[i]; }
    bool bad = false;
    for (int k = 0; k < g.nB; k++) {
        std::string s;
        char b[64];
        std::snprintf(b, sizeof b, wide ? "%5d" : "%4d", g.id[k]);
        s = b;
        pad(s, 5 + sh);
        s += "Bus";
        putf(s, 24 + sh, "%2.0f", (double)g.type[k], 2);
        putf(s, 27 + sh, "%6.4f", (g.type[k] >= 2) ? g.V0[k] : 1.0, 6);
        putf(s, 33 + sh, "%7.2f", (g.type[k] == 3) ? g.theta0[k] * 180.0 / PI_REF : 0.0, 7);
        putf(s, 40 + sh, "%9.3f", g.Pload[k] * g.baseMVA, 9);
        putf(s, 49 + sh, "%10.3f", g.Qload[k] * g.baseMVA, 10);
        putf(s, 59 + sh, "%8.3f", g.Pg[k] * g.baseMVA, 8);
        putf(s, 67 + sh, "%8.3f", g.Qg[k] * g.baseMVA, 8);
        putf(s, 76 + sh, "%7.1f", 100.0, 7);
        putf(s, 83 + sh, "%7.4f", (g.type[k] >= 2) ? g.V0[k] : 0.0, 7);
        putf(s, 90 + sh, "%7.2f", qmax[k] * g.baseMVA, 7);
        putf(s, 98 + sh, "%7.2f", qmin[k] * g.baseMVA, 7);
        putf(s, 106 + sh, "%8.4f", g.gsh[k], 8);
        putf(s, 114 + sh, "%8.4f", g.bsh[k], 8);
        s += "        0";
        if (s.find("-999") != std::string::npos) bad = true;
        std::fprintf(f, "%s\r\n", s.c_str());
    }
    std::fprintf(f, "-999\r\n");
    std::fprintf(f, "BRANCH DATA FOLLOWS                       %5d ITEMS\r\n", g.nL);
    for (int b = 0; b < g.nL; b++) {
        std::string s;
        char t[64];
        if (wide) std::snprintf(t, sizeof t, "%5d %5d", g.id[g.de[b] - 1], g.id[g.para[b] - 1]);
        else std::snprintf(t, sizeof t, "%4d %4d", g.id[g.de[b] - 1], g.id[g.para[b] - 1]);
        s = t;
        pad(s, 10 + 2 * sh);
        s += "1  1 1 0";
        const double a = std::hypot(g.tap_re[b], g.tap_im[b]);
        const bool is_tap = std::fabs(a - 1.0) > 1e-12 || g.phase[b] != 0.0;
        putf(s, 19 + 2 * sh, "%10.6f", g.r[b], 10);
        putf(s, 29 + 2 * sh, "%11.6f", g.x[b], 11);
        putf(s, 40 + 2 * sh, "%10.5f", g.bch[b], 10);
        putf(s, 76 + 2 * sh, "%6.4f", is_tap ? a : 0.0, 6);
        putf(s, 83 + 2 * sh, "%7.2f", g.phase[b] * 180.0 / PI_REF, 7);
        s += " 0.0    0.0     0.0    0.0   0.0";
        if (s.find("-999") != std::string::npos) bad = true;
        std::fprintf(f, "%s\r\n", s.c_str());
    }
    std::fprintf(f, "-999\r\n");
    std::fprintf(f, "LOSS ZONES FOLLOWS                     1 ITEMS\r\n  1 GBPF\r\n-99\r\n");
    std::fprintf(f, "INTERCHANGE DATA FOLLOWS                 0 ITEMS\r\n-9\r\n");
    std::fprintf(f, "TIE LINES FOLLOWS                     0 ITEMS\r\n-999\r\nEND OF DATA\r\n");
    std::fclose(f);
    if (bad) { set_error("a written line contains the section terminator -999"); return GBPF_E_INPUT; }
    return GBPF_OK;
}

// ---------------------------------------------------------------------------
// MATPOWER writer (rows read back by read_m above)
// ---------------------------------------------------------------------------

extern "C" gbpf_status gbpf_grid_write_m(const gbpf_grid *h, const char *path, const char *title) {
    if (!h || !path) return GBPF_E_ARG;
    const Grid &g = h->g;
    FILE *f = std::fopen(path, "wb");
    if (!f) { set_error(std::string("cannot write ") + path); return GBPF_E_INPUT; }
    const double base = g.baseMVA;
    auto row = [f](const std::vector<double> &v) {
        for (double x : v) std::fprintf(f, "\t%.17g", x);
        std::fprintf(f, ";\n");
    };
    std::fprintf(f, "function mpc = gbpf_case\n%%%s\n\n", title ? title : "synthetic grid");
    std::fprintf(f, "%%%% MATPOWER Case Format : Version 2\nmpc.version = '2';\n\n");
    std::fprintf(f, "%%%%-----  Power Flow Data  -----%%%%\n%%%% system MVA base\nmpc.baseMVA = %.17g;\n\n", base);
    std::fprintf(f, "%%%% bus data\n%%\tbus_i\ttype\tPd\tQd\tGs\tBs\tarea\tVm\tVa\tbaseKV\tzone\tVmax\tVmin\nmpc.bus = [\n");
    for (int k = 0; k < g.nB; k++) {
        const int t = g.type[k];
        const bool gen = t >= 2;
        // generation at a PQ bus folds into its load: the injection is kept
        const double pd = gen ? g.Pload[k] : g.Pload[k] - g.Pg[k];
        const double qd = gen ? g.Qload[k] : g.Qload[k] - g.Qg[k];
        row({(double)g.id[k], (double)(t <= 1 ? 1 : t), pd * base, qd * base, g.gsh[k] * base, g.bsh[k] * base, 1,
             g.V0[k], t == 3 ? g.theta0[k] * 180.0 / PI_REF : 0.0, g.Vbase[k], 1, 1.1, 0.9});
    }
    std::fprintf(f, "];\n\n%%%% generator data\n%%\tbus\tPg\tQg\tQmax\tQmin\tVg\tmBase\tstatus\tPmax\tPmin\tPc1\tPc2"
                    "\tQc1min\tQc1max\tQc2min\tQc2max\tramp_agc\tramp_10\tramp_30\tramp_q\tapf\nmpc.gen = [\n");
    std::vector<double> qmax(g.nB, 0), qmin(g.nB, 0);
    for (int i = 0; i < g.nPV; i++) { qmax[g.pv[i] - 1] = g.Qmax[i]; qmin[g.pv[i] - 1] = g.Qmin[i]; }
    for (int k = 0; k < g.nB; k++) {
        if (g.type[k] < 2) continue;
        const bool sl = g.type[k] == 3;
        std::vector<double> v = {(double)g.id[k], g.Pg[k] * base, g.Qg[k] * base, sl ? 9999.0 : qmax[k] * base,
                                 sl ? -9999.0 : qmin[k] * base, g.V0[k], base, 1, std::max(0.0, 2 * g.Pg[k] * base), 0};
        v.resize(21, 0.0);
        row(v);
    }
    std::fprintf(f, "];\n\n%%%% branch data\n%%\tfbus\ttbus\tr\tx\tb\trateA\trateB\trateC\tratio\tangle\tstatus"
                    "\tangmin\tangmax\nmpc.branch = [\n");
    for (int b = 0; b < g.nL; b++) {
        const double a = std::hypot(g.tap_re[b], g.tap_im[b]);
        const bool line = a == 1.0 && g.phase[b] == 0.0;
        row({(double)g.id[g.de[b] - 1], (double)g.id[g.para[b] - 1], g.r[b], g.x[b], g.bch[b], 0, 0, 0,
             line ? 0.0 : a, g.phase[b] * 180.0 / PI_REF, 1, -360, 360});
    }
    std::fprintf(f, "];\n");
    const bool ok = std::fclose(f) == 0;
    if (!ok) { set_error(std::string("cannot write ") + path); return GBPF_E_INPUT; }
    return GBPF_OK;
}

extern "C" int gbpf_grid_ybus_form(const gbpf_grid *h) { return h ? h->g.ybus_form : -1; }

extern "C" gbpf_status gbpf_grid_set_ybus_form(gbpf_grid *h, int form) {
    if (!h || (form != GBPF_YBUS_CDF && form != GBPF_YBUS_MATPOWER)) return GBPF_E_ARG;
    h->g.ybus_form = form;
    return GBPF_OK;
}

// ---------------------------------------------------------------------------
// Seeded synthetic grids
// ---------------------------------------------------------------------------

namespace {

// xoshiro256** seeded by splitmix64: portable, bit-identical on every host.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (int i = 0; i < 4; i++) {
            z += 0x9e3779b97f4a7c15ULL;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
            s[i] = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double u() { return (double)(next() >> 11) * 0x1.0p-53; }
    double u(double a, double b) { return a + (b - a) * u(); }
    int below(int n) { return (int)(u() * n); }
    double normal() {  // Marsaglia polar method
        for (;;) {
            double a = 2 * u() - 1, b = 2 * u() - 1, q = a * a + b * b;
            if (q > 0 && q < 1) return a * std::sqrt(-2 * std::log(q) / q);
        }
    }
    double lognormal_mean(double mean, double sigma) {  // E[X] = mean
        return std::exp(std::log(mean) - 0.5 * sigma * sigma + sigma * normal());
    }
    template <class T> void shuffle(std::vector<T> &v) {
        for (int i = (int)v.size() - 1; i > 0; i--) std::swap(v[i], v[below(i + 1)]);
    }
};

void alloc_buses(Grid &g, int n) {
    g = Grid();
    g.nB = n;
    g.baseMVA = 100.0;
    g.id.resize(n);
    std::iota(g.id.begin(), g.id.end(), 1);
    g.type.assign(n, 0);
    g.V0.assign(n, 1.0); g.theta0.assign(n, 0.0);
    g.Pload.assign(n, 0); g.Qload.assign(n, 0); g.Pg.assign(n, 0); g.Qg.assign(n, 0);
    g.gsh.assign(n, 0); g.bsh.assign(n, 0); g.Vbase.assign(n, 100.0);
}

void add_branch(Grid &g, int f, int t, double r, double x, double b, double tap) {
    g.de.push_back(f); g.para.push_back(t);
    g.r.push_back(r); g.x.push_back(x); g.bch.push_back(b);
    g.tap_re.push_back(tap); g.tap_im.push_back(0.0); g.phase.push_back(0.0);
    g.nL++;
}

void finish(Grid &g, const std::vector<double> &qlim, const std::vector<double> &vset) {
    g.rebuild_lists();
    g.Qmax.clear(); g.Qmin.clear(); g.Vset.clear();
    for (int i = 0; i < g.nPV; i++) {
        const int k = g.pv[i] - 1;
        g.Qmax.push_back(qlim[k]);
        g.Qmin.push_back(-qlim[k]);
        g.V0[k] = vset[k];
        g.Vset.push_back(vset[k]);
    }
}

// Ring over buses 1..n plus random chords up to nbr branches (configs 1 and 4).
void ring_chords(Rng &R, int n, int nbr, std::vector<std::pair<int, int>> &E) {
    std::vector<std::vector<char>> has(n, std::vector<char>(n, 0));
    for (int i = 0; i < n; i++) {
        int a = i, b = (i + 1) % n;
        E.push_back({std::min(a, b), std::max(a, b)});
        has[a][b] = has[b][a] = 1;
    }
    int guard = 0;
    while ((int)E.size() < nbr && guard++ < 100000) {
        int a = R.below(n), b = R.below(n);
        if (a == b || has[a][b]) continue;
        has[a][b] = has[b][a] = 1;
        E.push_back({std::min(a, b), std::max(a, b)});
    }
}

// Configs 1 and 4: ring-plus-chords grid of n buses; n == 14 is config 1
// exactly (impedances drawn per branch, PV output U(0.1,0.5)).  Scaled grids
// (config 4) dispatch every PV bus to the loads nearest to it and hand the
// drawn impedances to the branches by DC loading rank, as the 118-bus grid does.
std::vector<double> unit_dc_flows(int n, int slack, const std::vector<std::pair<int, int>> &E,
                                  const std::vector<double> &P, const std::vector<double> *X = nullptr);
void gen_ring_grid(uint64_t seed, int n, Grid &g) {
    Rng R(seed);
    alloc_buses(g, n);
    const bool c1 = (n == 14);
    const int nbr = c1 ? 20 : (int)std::lround(1.6 * n);
    const int npv = c1 ? 4 : std::max(1, (int)std::lround(R.u(0.2, 0.45) * (n - 1)));
    std::vector<std::pair<int, int>> E;
    ring_chords(R, n, nbr, E);
    const int ntr = c1 ? 3 : std::max(1, (int)std::lround(0.15 * nbr));
    std::vector<int> bidx(E.size());
    std::iota(bidx.begin(), bidx.end(), 0);
    R.shuffle(bidx);
    std::vector<char> is_tr(E.size(), 0);
    for (int i = 0; i < ntr && i < (int)bidx.size(); i++) is_tr[bidx[i]] = 1;
    std::vector<std::pair<double, double>> rx(E.size());
    for (auto &v : rx) { const double r = R.u(0.01, 0.08); v = {r, r * R.u(2, 5)}; }
    g.type[0] = 3;
    g.V0[0] = 1.06;
    std::vector<int> rest;
    for (int k = 1; k < n; k++) rest.push_back(k);
    R.shuffle(rest);
    std::vector<double> qlim(n, 0), vset(n, 1.0);
    for (int i = 0; i < n - 1; i++) g.type[rest[i]] = i < npv ? 2 : 0;
    for (int k = 1; k < n; k++) {
        if (g.type[k] == 2) {
            vset[k] = R.u(1.01, 1.09);
            g.Pg[k] = R.u(0.1, 0.5);
            qlim[k] = R.u(0.2, 0.5);
        } else {
            g.Pload[k] = R.u(0, 0.5);
            g.Qload[k] = g.Pload[k] * R.u(0.2, 0.5);
        }
    }
    if (!c1) {
        std::vector<std::vector<int>> nb(n);
        for (auto &e : E) { nb[e.first].push_back(e.second); nb[e.second].push_back(e.first); }
        std::vector<int> owner(n, -1), q;
        for (int k = 0; k < n; k++) if (g.type[k] == 2) { owner[k] = k; q.push_back(k); g.Pg[k] = 0; }
        for (size_t h = 0; h < q.size(); h++)
            for (int v : nb[q[h]]) if (owner[v] < 0) { owner[v] = owner[q[h]]; q.push_back(v); }
        for (int k = 0; k < n; k++) if (g.type[k] == 0 && owner[k] >= 0) g.Pg[owner[k]] += g.Pload[k];
        std::vector<double> Pinj(n);
        for (int k = 0; k < n; k++) Pinj[k] = g.Pg[k] - g.Pload[k];
        const std::vector<double> fl = unit_dc_flows(n, 0, E, Pinj);
        std::sort(rx.begin(), rx.end(), [](const std::pair<double, double> &a, const std::pair<double, double> &b) {
            return a.second < b.second;
        });
        std::vector<int> byflow(E.size());
        std::iota(byflow.begin(), byflow.end(), 0);
        std::stable_sort(byflow.begin(), byflow.end(), [&](int a, int b) { return fl[a] > fl[b]; });
        std::vector<std::pair<double, double>> zr(E.size());
        for (size_t i = 0; i < E.size(); i++) zr[byflow[i]] = rx[i];
        rx = zr;
    }
    for (size_t e = 0; e < E.size(); e++) {
        if (is_tr[e]) add_branch(g, E[e].first + 1, E[e].second + 1, rx[e].first, rx[e].second, 0.0, R.u(0.93, 0.98));
        else add_branch(g, E[e].first + 1, E[e].second + 1, rx[e].first, rx[e].second, R.u(0, 0.05), 0.0);
    }
    g.bsh[rest[npv + R.below(n - 1 - npv)]] = 0.19;  // one shunt on a PQ bus
    finish(g, qlim, vset);
}

// DC power flow with unit reactances (dense elimination; generator grids are
// small): |flow| per edge, used to give the smallest drawn impedances to the
// most loaded corridors so that the synthetic grid is planned, not random.
std::vector<double> unit_dc_flows(int n, int slack, const std::vector<std::pair<int, int>> &E,
                                  const std::vector<double> &P, const std::vector<double> *X) {
    const int m = n - 1;
    std::vector<int> ix(n, -1);
    for (int k = 0, c = 0; k < n; k++) if (k != slack) ix[k] = c++;
    std::vector<double> A((size_t)m * m, 0.0), b(m, 0.0);
    for (size_t q = 0; q < E.size(); q++) {
        const int a = ix[E[q].first], c = ix[E[q].second];
        const double y = X ? 1.0 / (*X)[q] : 1.0;
        if (a >= 0) A[(size_t)a * m + a] += y;
        if (c >= 0) A[(size_t)c * m + c] += y;
        if (a >= 0 && c >= 0) { A[(size_t)a * m + c] -= y; A[(size_t)c * m + a] -= y; }
    }
    for (int k = 0; k < n; k++) if (ix[k] >= 0) b[ix[k]] = P[k];
    for (int i = 0; i < m; i++) {  // symmetric positive definite: no pivoting
        const double p = A[(size_t)i * m + i];
        for (int r = i + 1; r < m; r++) {
            const double f = A[(size_t)r * m + i] / p;
            if (f == 0.0) continue;
            for (int c = i; c < m; c++) A[(size_t)r * m + c] -= f * A[(size_t)i * m + c];
            b[r] -= f * b[i];
        }
    }
    std::vector<double> th(m, 0.0);
    for (int i = m - 1; i >= 0; i--) {
        double acc = b[i];
        for (int c = i + 1; c < m; c++) acc -= A[(size_t)i * m + c] * th[c];
        th[i] = acc / A[(size_t)i * m + i];
    }
    std::vector<double> f(E.size());
    for (size_t e = 0; e < E.size(); e++) {
        const int a = ix[E[e].first], c = ix[E[e].second];
        f[e] = std::fabs((a >= 0 ? th[a] : 0.0) - (c >= 0 ? th[c] : 0.0)) / (X ? (*X)[e] : 1.0);
    }
    return f;
}

// Config 2: 118-bus meshed grid (1 slack, 53 PV, 64 PQ, 177 lines + 9
// transformers) on random planar-ish geometry: a minimum spanning tree of the
// 6-nearest-neighbour graph plus its shortest remaining edges.
void gen_118(uint64_t seed, Grid &g, int *slack_out) {
    Rng R(seed);
    const int n = 118, nbr = 186;
    alloc_buses(g, n);
    std::vector<double> px(n), py(n);
    for (int k = 0; k < n; k++) { px[k] = R.u(); py[k] = R.u(); }
    struct Cand { double d; int a, b; };
    std::vector<Cand> C;
    std::vector<std::vector<char>> seen(n, std::vector<char>(n, 0));
    for (int a = 0; a < n; a++) {
        std::vector<std::pair<double, int>> d;
        for (int b = 0; b < n; b++) if (b != a) d.push_back({std::hypot(px[a] - px[b], py[a] - py[b]), b});
        std::sort(d.begin(), d.end());
        for (int j = 0; j < 6; j++) {
            int b = d[j].second, lo = std::min(a, b), hi = std::max(a, b);
            if (!seen[lo][hi]) { seen[lo][hi] = 1; C.push_back({d[j].first, lo, hi}); }
        }
    }
    std::sort(C.begin(), C.end(), [](const Cand &x, const Cand &y) {
        return x.d != y.d ? x.d < y.d : (x.a != y.a ? x.a < y.a : x.b < y.b);
    });
    std::vector<int> uf(n);
    std::iota(uf.begin(), uf.end(), 0);
    std::function<int(int)> find = [&](int v) { return uf[v] == v ? v : uf[v] = find(uf[v]); };
    std::vector<std::pair<int, int>> E;
    std::vector<char> used(C.size(), 0);
    for (size_t i = 0; i < C.size(); i++) {
        int ra = find(C[i].a), rb = find(C[i].b);
        if (ra != rb) { uf[ra] = rb; E.push_back({C[i].a, C[i].b}); used[i] = 1; }
    }
    // connect leftover components (kNN graph may be disconnected)
    for (int k = 1; k < n; k++) {
        if (find(k) != find(0)) {
            int best = -1; double bd = 1e9;
            for (int j = 0; j < n; j++) if (find(j) == find(0)) {
                double d = std::hypot(px[k] - px[j], py[k] - py[j]);
                if (d < bd) { bd = d; best = j; }
            }
            uf[find(k)] = find(best);
            E.push_back({std::min(k, best), std::max(k, best)});
        }
    }
    // no bus hangs on a single branch: each leaf gets its shortest unused candidate
    {
        std::vector<int> dg(n, 0);
        for (auto &e : E) { dg[e.first]++; dg[e.second]++; }
        for (size_t i = 0; i < C.size() && (int)E.size() < nbr; i++) {
            if (used[i] || (dg[C[i].a] > 1 && dg[C[i].b] > 1)) continue;
            used[i] = 1;
            E.push_back({C[i].a, C[i].b});
            dg[C[i].a]++;
            dg[C[i].b]++;
        }
    }
    for (size_t i = 0; i < C.size() && (int)E.size() < nbr; i++) if (!used[i]) E.push_back({C[i].a, C[i].b});
    // bus types: slack = the best-connected bus, 53 PV, 64 PQ
    std::vector<int> deg(n, 0);
    for (auto &e : E) { deg[e.first]++; deg[e.second]++; }
    int slack = 0;
    for (int k = 1; k < n; k++) if (deg[k] > deg[slack]) slack = k;
    g.type[slack] = 3;
    g.V0[slack] = 1.05;
    std::vector<int> rest;
    for (int k = 0; k < n; k++) if (k != slack) rest.push_back(k);
    R.shuffle(rest);
    for (int i = 0; i < n - 1; i++) g.type[rest[i]] = i < 53 ? 2 : 0;
    std::vector<double> qlim(n, 0), vset(n, 1.0);
    double load = 0;
    for (int k = 0; k < n; k++) {
        if (k == slack) continue;
        if (g.type[k] == 0) {  // loads on the PQ buses
            g.Pload[k] = R.lognormal_mean(0.4, 0.6);
            g.Qload[k] = 0.35 * g.Pload[k];
            load += g.Pload[k];
        } else {
            vset[k] = R.u(1.0, 1.05);
            qlim[k] = R.u(0.1, 3.0);
        }
    }
    // Dispatch: each PQ bus is served by its nearest PV bus (multi-source BFS
    // over the branches); a PV bus generates the load it serves, so flows stay
    // local and the slack covers the losses.
    {
        std::vector<std::vector<int>> nb(n);
        for (auto &e : E) { nb[e.first].push_back(e.second); nb[e.second].push_back(e.first); }
        std::vector<int> owner(n, -1), q;
        for (int k = 0; k < n; k++) if (g.type[k] == 2) { owner[k] = k; q.push_back(k); }
        for (size_t h = 0; h < q.size(); h++)
            for (int v : nb[q[h]]) if (owner[v] < 0) { owner[v] = owner[q[h]]; q.push_back(v); }
        for (int k = 0; k < n; k++) if (g.type[k] == 0 && owner[k] >= 0) g.Pg[owner[k]] += g.Pload[k];
    }
    // 177 lines (R U(0.001,0.05), X = R U(3,8), B U(0,0.2)) and 9 transformers
    // (tap U(0.95,1.05)); drawn impedances go to edges by DC loading rank.
    std::vector<int> bidx(E.size());
    std::iota(bidx.begin(), bidx.end(), 0);
    R.shuffle(bidx);
    std::vector<char> is_tr(E.size(), 0);
    for (int i = 0; i < 9; i++) is_tr[bidx[i]] = 1;
    std::vector<double> Pinj(n);
    for (int k = 0; k < n; k++) Pinj[k] = g.Pg[k] - g.Pload[k];
    const std::vector<double> fl = unit_dc_flows(n, slack, E, Pinj);
    std::vector<std::pair<double, double>> rx(E.size());
    for (auto &v : rx) { const double r = R.u(0.001, 0.05); v = {r, r * R.u(3, 8)}; }
    std::sort(rx.begin(), rx.end(), [](const std::pair<double, double> &a, const std::pair<double, double> &b) {
        return a.second < b.second;
    });
    std::vector<int> byflow(E.size());
    std::iota(byflow.begin(), byflow.end(), 0);
    std::stable_sort(byflow.begin(), byflow.end(), [&](int a, int b) { return fl[a] > fl[b]; });
    std::vector<std::pair<double, double>> zr(E.size());
    for (size_t i = 0; i < E.size(); i++) zr[byflow[i]] = rx[i];
    for (size_t e = 0; e < E.size(); e++) {
        if (is_tr[e]) add_branch(g, E[e].first + 1, E[e].second + 1, zr[e].first, zr[e].second, 0.0, R.u(0.95, 1.05));
        else add_branch(g, E[e].first + 1, E[e].second + 1, zr[e].first, zr[e].second, R.u(0, 0.2), 0.0);
    }
    {  // the slack's Pg column carries the DC estimate of the losses, sum r f^2
        std::vector<double> xe(E.size());
        for (size_t e = 0; e < E.size(); e++) xe[e] = zr[e].second;
        const std::vector<double> f = unit_dc_flows(n, slack, E, Pinj, &xe);
        double loss = 0;
        for (size_t e = 0; e < E.size(); e++) loss += zr[e].first * f[e] * f[e];
        // reactive flows add about 0.25 % of the load on top of the DC losses
        g.Pg[slack] = loss + 0.0025 * load;
    }
    std::vector<int> all(n);
    std::iota(all.begin(), all.end(), 0);
    R.shuffle(all);
    for (int i = 0; i < 14; i++) g.bsh[all[i]] = R.u(-0.4, 0.4);
    finish(g, qlim, vset);
    if (slack_out) *slack_out = slack;
}

// Config 3 / 5: `tiles` copies of the 118-bus grid; copy t links to t+1 by 2
// ties and to one random earlier copy by 1 tie (R 0.01, X 0.05).  The middle
// copy keeps the only slack; the other copies' slacks become PV buses that
// generate their copy's estimated losses, so each copy is nearly balanced.
void gen_tiled(uint64_t seed, int tiles, Grid &g) {
    Rng R(seed ^ 0x5bd1e995ULL);
    Grid tg;
    const int nt = 118;
    alloc_buses(g, nt * tiles);
    std::vector<double> qlim(g.nB, 0), vset(g.nB, 1.0);
    std::vector<std::vector<int>> hubs(tiles);
    for (int t = 0; t < tiles; t++) {
        int sl = 0;
        gen_118(seed * 1000003ULL + (uint64_t)t * 7919ULL + 17ULL, tg, &sl);
        const int off = t * nt;
        {
            std::vector<int> pvs(tg.pv);
            std::stable_sort(pvs.begin(), pvs.end(), [&](int a, int b) { return tg.Pg[a - 1] > tg.Pg[b - 1]; });
            hubs[t].push_back(off + sl);
            for (int i = 0; i < 4 && i < (int)pvs.size(); i++) hubs[t].push_back(off + pvs[i] - 1);
            while (hubs[t].size() < 5) hubs[t].push_back(off + sl);
        }
        double tile_load = 0, tile_gen = 0;
        for (int k = 0; k < nt; k++) {
            const int K = off + k;
            g.type[K] = tg.type[k];
            g.Pload[K] = tg.Pload[k]; g.Qload[K] = tg.Qload[k];
            g.Pg[K] = tg.Pg[k]; g.Qg[K] = tg.Qg[k];
            g.gsh[K] = tg.gsh[k]; g.bsh[K] = tg.bsh[k];
            tile_load += tg.Pload[k];
            if (k != sl) tile_gen += tg.Pg[k];
        }
        for (int i = 0; i < tg.nPV; i++) {
            const int K = off + tg.pv[i] - 1;
            qlim[K] = tg.Qmax[i];
            vset[K] = tg.Vset[i];
        }
        for (int b = 0; b < tg.nL; b++)
            add_branch(g, off + tg.de[b], off + tg.para[b], tg.r[b], tg.x[b], tg.bch[b], tg.tap_re[b]);
        const int K = off + sl;
        if (t == tiles / 2) {  // the middle copy keeps the slack: tie flows split both ways
            g.V0[K] = tg.V0[sl];
        } else {
            g.type[K] = 2;
            vset[K] = tg.V0[sl];
            qlim[K] = 3.0;
            g.Pg[K] = std::max(0.0, tile_load - tile_gen) + tg.Pg[sl];  // the copy's losses
        }
    }
    // Ties join generator hubs (a copy's former slack and its four largest PV
    // units), as tiled IEEE cases join generator buses: copy t to t+1 by the
    // two former slacks and by two random hubs, and to one random earlier copy
    // by two random hubs.
    for (int t = 0; t + 1 < tiles; t++) {
        add_branch(g, hubs[t][0] + 1, hubs[t + 1][0] + 1, 0.01, 0.05, 0.0, 0.0);
        add_branch(g, hubs[t][1 + R.below(4)] + 1, hubs[t + 1][1 + R.below(4)] + 1, 0.01, 0.05, 0.0, 0.0);
        const int u = R.below(t + 1);
        add_branch(g, hubs[u][R.below(5)] + 1, hubs[t + 1][R.below(5)] + 1, 0.01, 0.05, 0.0, 0.0);
    }
    finish(g, qlim, vset);
}

}  // namespace

extern "C" gbpf_status gbpf_generate(int kind, unsigned long long seed, int tiles, int nbus,
                                     gbpf_grid **out) {
    if (!out) return GBPF_E_ARG;
    *out = nullptr;
    auto *h = new gbpf_grid;
    switch (kind) {
    case 1: gen_ring_grid(seed, 14, h->g); break;
    case 2: gen_118(seed, h->g, nullptr); break;
    case 3:
        if (tiles < 1 || tiles > 4096) { delete h; return GBPF_E_ARG; }
        gen_tiled(seed, tiles, h->g);
        break;
    case 4:
        if (nbus < 3 || nbus > 100000) { delete h; return GBPF_E_ARG; }
        gen_ring_grid(seed, nbus, h->g);
        break;
    default: delete h; return GBPF_E_ARG;
    }
    // tap convention of the reader: a == 0 in the file means "no transformer"
    Grid &g = h->g;
    for (int b = 0; b < g.nL; b++) if (g.tap_re[b] == 0.0) g.tap_re[b] = 1.0;
    *out = h;
    return GBPF_OK;
}
