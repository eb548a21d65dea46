// sc_input.cpp -- readers for options / top.init / config.init and the derived
// interaction table.  See sc_input.h for the reference functions each part follows.

#include "sc_input.h"

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>

namespace scg {

namespace {

const double kPI = 3.141592653589793238462643383279;   // macros.h:63
const double kPIH = 1.57079632679489661923132169163975;
const double kDEGTORAD = 0.017453292519943295769236907683;
const double kZEROTOL = 1.0e-12;

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r' || s[a] == '\n')) ++a;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r' || s[b - 1] == '\n')) --b;
    return s.substr(a, b - a);
}
std::string stripComment(const std::string& s) {
    size_t k = s.find('#');
    return k == std::string::npos ? s : s.substr(0, k);
}
std::vector<std::string> lines(const std::string& text) {
    std::vector<std::string> out;
    std::string cur;
    for (char ch : text) {
        if (ch == '\n') { out.push_back(cur); cur.clear(); }
        else cur.push_back(ch);
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}
bool parseLong(const std::string& s, long& v) {
    char* end = nullptr;
    v = std::strtol(s.c_str(), &end, 10);
    return end != s.c_str() && *end == 0;
}
bool parseDouble(const std::string& s, double& v) {
    char* end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end != s.c_str() && *end == 0;
}
std::vector<std::string> words(const std::string& s) {
    std::istringstream is(s);
    std::vector<std::string> w;
    std::string x;
    while (is >> x) w.push_back(x);
    return w;
}
std::string upper(std::string s) {
    for (auto& c : s) c = (char)std::toupper((unsigned char)c);
    return s;
}
// beforecommand / aftercommand of scOOP/mc/simlib.cpp: text before / after the first separator.
std::string before(const std::string& s, char c) {
    size_t k = s.find(c);
    return trim(k == std::string::npos ? s : s.substr(0, k));
}
std::string after(const std::string& s, char c) {
    size_t k = s.find(c);
    return trim(k == std::string::npos ? s : s.substr(k + 1));
}

int convertGeotype(const std::string& g) {   // Inicializer::convertGeotype (inicializer.cpp:855-885)
    static const struct { const char* n; int v; } tab[] = {
        {"SCN", SCN}, {"SCA", SCA}, {"PSC", PSC}, {"CPSC", CPSC}, {"CHPSC", CHPSC}, {"CHCPSC", CHCPSC},
        {"TPSC", TPSC}, {"TCPSC", TCPSC}, {"TCHPSC", TCHPSC}, {"TCHCPSC", TCHCPSC}, {"SP", SP}, {"SPN", SPN},
        {"SPA", SPA}};
    for (auto& e : tab) if (g == e.n) return e.v;
    return 0;
}

inline double dot(const Vec3& a, const Vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double vsize(const Vec3& v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
inline void normalise(Vec3& v) {
    double t = vsize(v);
    if (t != 0.0) { t = 1.0 / t; v.x *= t; v.y *= t; v.z *= t; }
}
inline void orthogonalise(Vec3& a, const Vec3& b) {
    double dp = dot(a, b);
    a.x -= dp * b.x; a.y -= dp * b.y; a.z -= dp * b.z;
}
inline void rotateAbout(Vec3& v, const Vec3& axis, double c, double s) {   // Vector::rotate (Vector.h:133-157)
    double qw = c, qx = axis.x * s, qy = axis.y * s, qz = axis.z * s;
    double t2 = qw * qx, t3 = qw * qy, t4 = qw * qz, t5 = -qx * qx, t6 = qx * qy, t7 = qx * qz, t8 = -qy * qy,
           t9 = qy * qz, t10 = -qz * qz;
    double nx = 2.0 * ((t8 + t10) * v.x + (t6 - t4) * v.y + (t3 + t7) * v.z) + v.x;
    double ny = 2.0 * ((t4 + t6) * v.x + (t5 + t10) * v.y + (t9 - t2) * v.z) + v.y;
    double nz = 2.0 * ((t7 - t3) * v.x + (t2 + t9) * v.y + (t5 + t8) * v.z) + v.z;
    v = {nx, ny, nz};
}

// One [Types] line (Inicializer::fillTypes, inicializer.cpp:660-852).
int fillType(Topology& t, const std::string& line, std::string& err) {
    std::vector<std::string> w = words(after(line, ':'));
    if (w.size() < 3) { err = "top.init: bad type line: " + line; return -1; }
    long type;
    if (!parseLong(w[1], type) || type < 0 || type >= MAXT) { err = "top.init: bad type number: " + line; return -1; }
    int g = convertGeotype(w[2]);
    if (!g) { err = "top.init: unknown GEOTYPE " + w[2]; return -1; }
    double param[12] = {0};
    int n = 0;
    for (size_t k = 3; k < w.size() && n < 12; ++k, ++n)
        if (!parseDouble(w[k], param[n])) break;
    int fields = n - 2;
    auto need = [&](bool cond, const char* what) {
        if (cond) { err = std::string("top.init: wrong number of parameters for ") + w[2] + " (" + what + ")"; return true; }
        return false;
    };
    if (need(g == SPN && fields != 0, "EPSILON SIGMA")) return -1;
    if (need(g == SCN && fields != 1, "EPSILON SIGMA SC_LENGTH")) return -1;
    if (need(g == SPA && fields != 2, "EPSILON SIGMA ATTRACT_DIST ATTRACT_SWITCH")) return -1;
    if (need(g == SCA && fields != 3, "EPSILON SIGMA ATTRACT_DIST ATTRACT_SWITCH SC_LENGTH")) return -1;
    if (need((g == PSC || g == CPSC) && fields != 6, "... PATCH_ANGLE PATCH_SWITCH SC_LENGTH PARALLEL_EPS")) return -1;
    if (need((g == CHPSC || g == CHCPSC) && fields != 7, "... PARALLEL_EPS CHIRAL_ANGLE")) return -1;
    if (need((g == TPSC || g == TCPSC) && fields != 9, "... PATCH_ROTATION PATCH_ANGLE PATCH_SWITCH")) return -1;
    if (need((g == TCHPSC || g == TCHCPSC) && fields != 10, "... PATCH_SWITCH CHIRAL_ANGLE")) return -1;
    IaParam& p = t.ia[type][type];
    p.geotype[0] = p.geotype[1] = g;
    p.epsilon = param[0];
    p.sigma = param[1];
    p.sigmaSq = p.sigma * p.sigma;
    p.A = 4 * p.epsilon * pow(p.sigma, 12);
    p.B = 4 * p.epsilon * pow(p.sigma, 6);
    p.rcutwca = (p.sigma) * pow(2.0, 1.0 / 6.0);
    p.rcutwcaSq = p.rcutwca * p.rcutwca;
    if (fields > 0 && fields != 1 && fields != 3) {
        p.pdis = param[2];
        p.pdisSq = p.pdis * p.pdis;
        p.pswitch = param[3];
        p.pswitchINV = 1.0 / param[3];
        p.rcut = (g != SPN) ? p.pswitch + p.pdis : 0.0;
        p.rcutSq = p.rcut * p.rcut;
    }
    if (fields == 1) for (int i = 0; i < 2; ++i) { p.len[i] = param[2]; p.half_len[i] = param[2] / 2; }
    if (fields == 3) for (int i = 0; i < 2; ++i) { p.len[i] = param[4]; p.half_len[i] = param[4] / 2; }
    if (fields > 2 && fields != 3) {
        for (int i = 0; i < 2; ++i) {
            p.len[i] = param[6];
            p.half_len[i] = param[6] / 2;
            p.pangl[i] = param[4];
            p.panglsw[i] = param[5];
            p.pcangl[i] = cos(param[4] / 2.0 / 180 * kPI);
            p.pcanglsw[i] = cos((param[4] / 2.0 + param[5]) / 180 * kPI);
            p.pcoshalfi[i] = cos((param[4] / 2.0 + param[5]) / 2.0 / 180 * kPI);
            p.psinhalfi[i] = sqrt(1.0 - p.pcoshalfi[i] * p.pcoshalfi[i]);
            p.parallel = param[7];
        }
    }
    if (fields == 7) for (int i = 0; i < 2; ++i) {
        p.chiral_cos[i] = cos(param[8] / 360 * kPI);
        p.chiral_sin[i] = sqrt(1 - p.chiral_cos[i] * p.chiral_cos[i]);
    }
    if (fields == 9 || fields == 10) for (int i = 0; i < 2; ++i) {
        p.csecpatchrot[i] = cos(param[8] / 360 * kPI);
        p.ssecpatchrot[i] = sqrt(1 - p.csecpatchrot[i] * p.csecpatchrot[i]);
        p.pangl[i + 2] = param[9];
        p.panglsw[i + 2] = param[10];
        p.pcangl[i + 2] = cos(param[9] / 2.0 / 180 * kPI);
        p.pcanglsw[i + 2] = cos((param[9] / 2.0 + param[10]) / 180 * kPI);
        p.pcoshalfi[i + 2] = cos((param[9] / 2.0 + param[10]) / 2.0 / 180 * kPI);
        p.psinhalfi[i + 2] = sqrt(1.0 - p.pcoshalfi[i + 2] * p.pcoshalfi[i + 2]);
    }
    if (fields == 10) for (int i = 0; i < 2; ++i) {
        p.chiral_cos[i] = cos(param[11] / 360 * kPI);
        p.chiral_sin[i] = sqrt(1 - p.chiral_cos[i] * p.chiral_cos[i]);
    }
    if (g < SP)
        p.volume = 4.0 / 3.0 * kPI * pow((p.sigma) / 2.0, 3.0) + kPI / 2.0 * p.len[0] * pow((p.sigma) / 2.0, 2.0);
    else
        p.volume = 4.0 / 3.0 * kPI * pow((p.sigma) / 2.0, 3.0);
    if (p.rcutwca > t.sqmaxcut) t.sqmaxcut = p.rcutwca;
    if (p.rcut > t.sqmaxcut) t.sqmaxcut = p.rcut;
    return 0;
}

// One line inside a molecule block (Inicializer::fillMol, inicializer.cpp:929-1108).
int fillMolLine(MolType& m, const std::string& cmdIn, const std::string& params, std::string& err) {
    std::string cmd = upper(trim(cmdIn));
    std::vector<std::string> w = words(params);
    if (cmd == "PARTICLES") {
        // "TYPE [SWITCHTYPE DELTA_MU]" (inicializer.cpp:955-985): one field, or three
        long ty, sw = -1;
        double dmu = 0.0;
        if (w.empty() || !parseLong(w[0], ty)) { err = "top.init: could not read a particle"; return -1; }
        if (w.size() >= 2) {
            if (w.size() < 3 || !parseLong(w[1], sw) || !parseDouble(w[2], dmu)) {
                err = "top.init: could not read a particle"; return -1;
            }
            if (sw < 0 || sw >= MAXT) { err = "top.init: switch type out of range"; return -1; }
        }
        if (ty < 0) { err = "top.init: particles include negative type"; return -1; }
        if (ty > MAXT) { err = "top.init: particle type out of range"; return -1; }
        m.types.push_back((int)ty);
        m.switchTypes.push_back((int)sw);
        m.deltaMu.push_back(dmu);
        return 0;
    }
    double k = 0, eq = 0;
    auto two = [&](const char* what) {
        if (w.size() < 2 || !parseDouble(w[0], k) || !parseDouble(w[1], eq)) {
            err = std::string("top.init: wrong number of parameters for ") + what;
            return false;
        }
        if (eq < 0) { err = std::string("top.init: ") + what + " equilibrium value cannot be negative"; return false; }
        return true;
    };
    if (cmd == "BOND1") { if (!two("bond1")) return -1; m.bond1c = k; m.bond1eq = eq; return 0; }
    if (cmd == "BOND2") { if (!two("bond2")) return -1; m.bond2c = k; m.bond2eq = eq; return 0; }
    if (cmd == "BONDD") { if (!two("bondd")) return -1; m.bonddc = k; m.bonddeq = eq; return 0; }
    if (cmd == "BONDH") { if (!two("bondh")) return -1; m.bondhc = k; m.bondheq = eq; return 0; }
    if (cmd == "ANGLE1") { if (!two("angle1")) return -1; m.angle1c = k; m.angle1eq = eq * kDEGTORAD; return 0; }
    if (cmd == "ANGLE2") { if (!two("angle2")) return -1; m.angle2c = k; m.angle2eq = eq * kDEGTORAD; return 0; }
    if (cmd == "ACTIVITY") {
        // inicializer.cpp:1087-1096; the options' nGrandCanon is checked against it once
        // both files are read (Context::setup), chemPot = log(activity Nav 1e-24) there
        if (w.empty() || !parseDouble(w[0], k)) { err = "top.init: could not read the activity"; return -1; }
        m.activity = k;
        return 0;
    }
    err = "top.init: unknown molecule parameter: " + cmd;
    return -1;
}

}  // namespace

double anInt(double d) {
    // Cuboid::image takes the low 32 bits of d + 1.5*2^52 as an int
    // (geometry.h:110-128): round-half-even for |d| < 2^31.
    volatile double t = d + 6755399441055744.0;
    double tt = t;
    uint64_t bits;
    std::memcpy(&bits, &tt, 8);
    return (double)(int32_t)(uint32_t)(bits & 0xffffffffu);
}

Vec3 image(const Vec3& r1, const Vec3& r2, const Vec3& box) {
    double dx = r1.x - r2.x, dy = r1.y - r2.y, dz = r1.z - r2.z;
    return {box.x * (dx - anInt(dx)), box.y * (dy - anInt(dy)), box.z * (dz - anInt(dz))};
}

int readOptionsText(const std::string& text, Options& o, std::string& err) {
    struct Opt { const char* id; char kind; void* var; bool optional; bool set; };
    double transmx = 0, rotmx = 0, chainmmx = 0, chainrmx = 0;
    std::vector<std::pair<int, double>> transType;
    Opt opts[] = {
        {"write_cluster", 'L', &o.write_cluster, false, false}, {"adjust", 'L', &o.adjust, false, false},
        {"movie", 'L', &o.movie, false, false}, {"nequil", 'L', &o.nequil, false, false},
        {"nsweeps", 'L', &o.nsweeps, false, false}, {"nrepchange", 'L', &o.nrepchange, false, false},
        {"nGrandCanon", 'L', &o.nGrandCanon, false, false}, {"nClustMove", 'L', &o.nClustMove, false, false},
        {"paramfrq", 'L', &o.paramfrq, false, false}, {"report", 'L', &o.report, false, false},
        {"seed", 'L', &o.seed, false, false}, {"pairlist_update", 'I', &o.pairlist_update, false, false},
        {"ptype", 'I', &o.ptype, false, false}, {"wlm", '2', &o.wlm, false, false},
        {"wlmtype", 'I', &o.wlmtype, false, false}, {"press", 'D', &o.press, false, false},
        {"paralpress", 'D', &o.paralpress, false, false}, {"edge_mx", 'D', &o.edge_mx, false, false},
        {"shave", 'D', &o.shave, false, false}, {"chainprob", 'D', &o.chainprob, false, false},
        {"switchprob", 'D', &o.switchprob, false, false}, {"temper", 'D', &o.temper, false, false},
        {"paraltemper", 'D', &o.paraltemper, false, false}, {"transmx", 'D', &transmx, false, false},
        {"transmx_type", 'T', nullptr, true, false}, {"rotmx", 'D', &rotmx, false, false},
        {"coneAngle", 'D', &o.coneAngle, true, false}, {"chainmmx", 'D', &chainmmx, false, false},
        {"chainrmx", 'D', &chainrmx, false, false},
    };
    for (const std::string& raw : lines(text)) {
        std::string line = trim(stripComment(raw));
        if (line.empty()) continue;
        size_t eq = line.find('=');
        if (eq == std::string::npos) { err = "options: error parsing line (" + line + ")"; return -1; }
        std::string id = trim(line.substr(0, eq));
        std::string rest = line.substr(eq + 1);
        size_t eq2 = rest.find('=');
        std::string value = trim(eq2 == std::string::npos ? rest : rest.substr(0, eq2));
        if (value.empty()) { err = "options: error parsing line (" + line + ")"; return -1; }
        Opt* hit = nullptr;
        for (auto& op : opts) if (id == op.id) { hit = &op; break; }
        if (!hit) { std::fprintf(stderr, "options: unknown identifier %s, ignored\n", id.c_str()); continue; }
        bool ok = true;
        if (hit->kind == 'L') { long v; ok = parseLong(value, v); *(long*)hit->var = v; }
        else if (hit->kind == 'I') { long v; ok = parseLong(value, v); *(int*)hit->var = (int)v; }
        else if (hit->kind == 'D') { double v; ok = parseDouble(value, v); *(double*)hit->var = v; }
        else if (hit->kind == '2') {
            std::vector<std::string> w = words(value);
            long a = 0, b = 0;
            ok = !w.empty() && w.size() <= 2 && parseLong(w[0], a) && (w.size() < 2 || parseLong(w[1], b));
            ((int*)hit->var)[0] = (int)a;
            ((int*)hit->var)[1] = (int)b;
        } else if (hit->kind == 'T') {
            std::vector<std::string> w = words(value);
            for (size_t k = 0; k + 1 < w.size(); k += 2) {
                long ty; double v;
                if (!parseLong(w[k], ty) || !parseDouble(w[k + 1], v) || ty < 0 || ty >= MAXT) { ok = false; break; }
                transType.push_back({(int)ty, v});
            }
        }
        if (!ok) { err = "options: could not convert value of " + id + " (" + value + ")"; return -1; }
        hit->set = true;
    }
    for (auto& op : opts)
        if (!op.set && !op.optional) { err = std::string("options: option '") + op.id + "' is not set"; return -1; }
    if (rotmx < 0.0 || rotmx > 180) { err = "options: maximum orientation change must be in range 0 to 180"; return -1; }
    if (chainrmx < 0.0 || chainrmx > 180) { err = "options: maximum chain orientation change must be in range 0 to 180"; return -1; }
    if (o.ptype < 0 || o.ptype > 5) { err = "options: unknown pressure coupling"; return -1; }
    if (o.wlm[0] < 0 || o.wlm[0] > 9 || o.wlm[1] < 0 || o.wlm[1] > 9) { err = "options: unknown Wang-Landau method"; return -1; }
    o.rotmx_deg = rotmx;
    o.chainrmx_deg = chainrmx;
    o.rot_angle = rotmx / 180.0 * kPIH * 0.5;   // sim.h:359
    o.chain_angle = chainrmx / 180.0 * kPIH;    // sim.h:361
    o.edge_mx *= 2.0;                           // sim.h:363-366
    o.transmx = transmx * 2.0;
    o.chainmmx = chainmmx * 2.0;
    o.coneAngle *= kDEGTORAD;
    for (int i = 0; i < MAXT; ++i) o.trans_type[i] = o.transmx;
    for (auto& tt : transType) o.trans_type[tt.first] = tt.second;
    return 0;
}

int readTopologyText(const std::string& text, Topology& t, std::string& err) {
    std::string key;
    int curMol = -1;
    std::vector<std::string> ls = lines(text);
    for (size_t li = 0; li < ls.size(); ++li) {
        std::string line = ls[li];
        // line continuation with a trailing backslash (simlib.cpp continuing)
        while (!trim(line).empty() && trim(line).back() == '\\' && li + 1 < ls.size()) {
            std::string tl = trim(line);
            line = tl.substr(0, tl.size() - 1) + ls[++li];
        }
        line = trim(stripComment(line));
        if (line.empty()) continue;
        if (line[0] == '[') {
            key = upper(before(line.substr(1), ']'));
            continue;
        }
        if (key == "TYPES") {
            if (fillType(t, line, err)) return -1;
        } else if (key == "MOLECULES") {
            if (curMol < 0) {
                std::string name = before(line, ':');
                t.mols.push_back(MolType());
                t.mols.back().name = name;
                curMol = (int)t.mols.size() - 1;
            }
            // fillMol: the text between '{' and '}' of this line is one command
            std::string body = after(before(line, '}'), '{');
            if (!body.empty()) {
                if (fillMolLine(t.mols[curMol], before(body, ':'), after(body, ':'), err)) return -1;
            }
            if (line.find('}') != std::string::npos) curMol = -1;
        } else if (key == "SYSTEM") {
            std::vector<std::string> w = words(line);
            long cnt;
            if (w.size() < 2 || !parseLong(w[1], cnt)) { err = "top.init: failed reading system from (" + line + ")"; return -1; }
            t.system.push_back({w[0], cnt});
        } else if (key == "EXCLUDE") {
            std::vector<std::string> w = words(line);
            if (w.size() % 2) { err = "top.init: exclusions need pairs of types"; return -1; }
            for (size_t k = 0; k < w.size(); k += 2) {
                long a, b;
                if (!parseLong(w[k], a) || !parseLong(w[k + 1], b) || a < 0 || b < 0 || a >= MAXT || b >= MAXT) {
                    err = "top.init: bad exclusion"; return -1;
                }
                t.exclusions[a][b] = t.exclusions[b][a] = true;
            }
        } else if (key == "EXTER" || key == "POOL") {
            err = "top.init: [" + key + "] (external wall / grand-canonical pool) is outside the GPU hot path";
            return -1;
        } else {
            err = "top.init: invalid keyword " + key;
            return -1;
        }
    }
    for (auto& m : t.mols) {
        if ((m.bond1c > 0.0 && m.bonddc > 0.0) || (m.bondhc > 0.0 && m.bonddc > 0.0) || (m.bond1c > 0.0 && m.bondhc > 0.0)) {
            err = "top.init: defined bond1, bondh or bondd, choose only one"; return -1;
        }
        if ((int)m.types.size() > MAXCHL) { err = "top.init: molecule longer than MAXCHL"; return -1; }
        for (int ty : m.types)
            if (t.ia[ty][ty].geotype[0] == 0) { err = "top.init: molecule uses an undefined type"; return -1; }
        for (int ty : m.switchTypes)
            if (ty >= 0 && t.ia[ty][ty].geotype[0] == 0) { err = "top.init: molecule uses an undefined switch type"; return -1; }
    }
    // Topo::genParamPairs (topo.cpp:5-138)
    double length = 0;
    for (int i = 0; i < MAXT; ++i) {
        for (int j = 0; j < MAXT; ++j) {
            if (i == j) continue;
            if (t.ia[j][j].geotype[0] == 0 || t.ia[i][i].geotype[0] == 0) continue;
            IaParam& p = t.ia[i][j];
            const IaParam& di = t.ia[i][i];
            const IaParam& dj = t.ia[j][j];
            int a[2] = {i, j};
            for (int k = 0; k < 2; ++k) {
                const IaParam& dk = t.ia[a[k]][a[k]];
                p.geotype[k] = dk.geotype[0];
                p.len[k] = dk.len[0];
                if (dk.len[0] > 0) {
                    if (length == 0) length = dk.len[0];
                    else if (length > 0 && length != dk.len[0]) {
                        err = "top.init: different lengths for spherocylinders are not supported (topo.cpp:25-32)";
                        return -1;
                    }
                }
                p.half_len[k] = dk.half_len[0];
                if (p.geotype[k] >= PSC && p.geotype[k] < SP) {
                    p.pangl[k] = dk.pangl[0];
                    p.panglsw[k] = dk.panglsw[0];
                    p.pcangl[k] = cos(p.pangl[k] / 2.0 / 180 * kPI);
                    p.pcanglsw[k] = cos((p.pangl[k] / 2.0 + p.panglsw[k]) / 180 * kPI);
                    p.pcoshalfi[k] = cos((p.pangl[k] / 2.0 + p.panglsw[k]) / 2.0 / 180 * kPI);
                    p.psinhalfi[k] = sqrt(1.0 - p.pcoshalfi[k] * p.pcoshalfi[k]);
                }
                if (isChiral(p.geotype[k])) { p.chiral_cos[k] = dk.chiral_cos[0]; p.chiral_sin[k] = dk.chiral_sin[0]; }
                if (isTwoPatch(p.geotype[k])) {
                    p.csecpatchrot[k] = dk.csecpatchrot[0];
                    p.ssecpatchrot[k] = dk.ssecpatchrot[0];
                    p.pangl[k + 2] = dk.pangl[2];
                    p.panglsw[k + 2] = dk.panglsw[2];
                    p.pcangl[k + 2] = cos(p.pangl[k + 2] / 2.0 / 180 * kPI);
                    p.pcanglsw[k + 2] = cos((p.pangl[k + 2] / 2.0 + p.panglsw[k + 2]) / 180 * kPI);
                    p.pcoshalfi[k + 2] = cos((p.pangl[k + 2] / 2.0 + p.panglsw[k + 2]) / 2.0 / 180 * kPI);
                    p.psinhalfi[k + 2] = sqrt(1.0 - p.pcoshalfi[k + 2] * p.pcoshalfi[k + 2]);
                }
            }
            p.sigma = ((di.sigma + dj.sigma) * 0.5);
            p.sigmaSq = p.sigma * p.sigma;
            p.epsilon = sqrt(di.epsilon * dj.epsilon);
            p.A = 4 * p.epsilon * pow(p.sigma, 12);
            p.B = 4 * p.epsilon * pow(p.sigma, 6);
            p.pswitch = ((di.pswitch + dj.pswitch) * 0.5);
            p.pswitchINV = 1.0 / p.pswitch;
            p.rcutwca = (p.sigma) * pow(2.0, 1.0 / 6.0);
            p.rcutwcaSq = p.rcutwca * p.rcutwca;
            if ((di.parallel > 0) && (dj.parallel > 0)) p.parallel = sqrt(di.parallel * dj.parallel);
            if ((di.parallel < 0) && (dj.parallel < 0)) p.parallel = -sqrt(di.parallel * dj.parallel);
            p.pdis = (((di.pdis - di.rcutwca) + (dj.pdis - dj.rcutwca)) * 0.5) + p.rcutwca;
            p.pdisSq = p.pdis * p.pdis;
            p.rcut = (p.geotype[0] == SPN || p.geotype[1] == SPN) ? 0.0 : p.pswitch + p.pdis;
            p.rcutSq = p.rcut * p.rcut;
            if (p.rcutwca > t.sqmaxcut) t.sqmaxcut = p.rcutwca;
            if (p.rcut > t.sqmaxcut) t.sqmaxcut = p.rcut;
        }
    }
    for (int i = 0; i < MAXT; ++i)
        for (int j = 0; j < MAXT; ++j) t.ia[i][j].exclude = t.exclusions[i][j];
    // Topo::genTopoParams (topo.cpp:140-153)
    double maxlength = 0;
    for (int i = 0; i < MAXT; ++i) if (maxlength < t.ia[i][i].len[0]) maxlength = t.ia[i][i].len[0];
    t.sqmaxcut += maxlength;
    t.sqmaxcut *= 1.1;
    t.maxcut = t.sqmaxcut;
    t.sqmaxcut = t.sqmaxcut * t.sqmaxcut;
    return 0;
}

int buildParticles(const Topology& t, Config& c, std::string& err) {
    c.p.clear();
    for (auto& sys : t.system) {
        int mol = -1;
        for (size_t m = 0; m < t.mols.size(); ++m) if (t.mols[m].name == sys.first) { mol = (int)m; break; }
        if (mol < 0) { err = "top.init: molecule " + sys.first + " is not defined"; return -1; }
        for (long j = 0; j < sys.second; ++j)
            for (size_t k = 0; k < t.mols[mol].types.size(); ++k) {
                Particle p;
                p.type = t.mols[mol].types[k];
                p.switchtype = t.mols[mol].switchTypes[k];   // setParticlesParams, inicializer.cpp:428-431
                p.molType = mol;
                c.p.push_back(p);
            }
    }
    // Inicializer::initGroupLists (inicializer.cpp:330-397)
    c.molTypeCount = (int)t.mols.size();
    c.first.assign(c.molTypeCount + 1, 0);
    int N = (int)c.p.size(), i = 0;
    for (int type = 0; type < c.molTypeCount; ++type) {
        bool empty = true;
        while (i < N) {
            if (type == c.p[i].molType) {
                c.first[type] = i;
                int count = 0;
                for (int j = i; j < N; ++j) if (type == c.p[j].molType) ++count;
                for (int j = type + 1; j < c.molTypeCount; ++j) c.first[j] = i + count;
                empty = false;
                break;
            }
            ++i;
        }
        if (empty) i = c.first[type];
    }
    c.first[c.molTypeCount] = N;
    // the move kernels assume every molecule type sits in one contiguous run
    for (int k = 0; k < N; ++k) {
        int m = c.p[k].molType;
        if (k < c.first[m] || k >= c.first[m + 1]) { err = "top.init: [System] must list each molecule type in one block"; return -1; }
    }
    return 0;
}

int readConfigText(const std::string& text, const Topology& t, Config& c, std::string& err) {
    std::vector<std::string> ls = lines(text);
    size_t li = 0;
    // first non-empty line: the box (Inicializer::initConfig, inicializer.cpp:103-147)
    while (li < ls.size() && trim(stripComment(ls[li])).empty()) ++li;
    if (li >= ls.size()) { err = "config.init: could not read box size"; return -1; }
    {
        std::string l = trim(stripComment(ls[li++]));
        if (std::sscanf(l.c_str(), "%le %le %le", &c.box.x, &c.box.y, &c.box.z) != 3) {
            std::string l2 = after(l, 'x');
            if (std::sscanf(l2.c_str(), "%le %le %le", &c.box.x, &c.box.y, &c.box.z) != 3) {
                err = "config.init: could not read box size"; return -1;
            }
        }
    }
    for (size_t i = 0; i < c.p.size(); ++i) {
        if (li >= ls.size()) { err = "config.init: fewer particle lines than [System] declares"; return -1; }
        std::string l = trim(stripComment(ls[li++]));
        Particle& p = c.p[i];
        int sw = 0;
        int fields = std::sscanf(l.c_str(), "%le %le %le %le %le %le %le %le %le %d", &p.pos.x, &p.pos.y, &p.pos.z,
                                 &p.dir.x, &p.dir.y, &p.dir.z, &p.pd[0].x, &p.pd[0].y, &p.pd[0].z, &sw);
        p.pd[1] = {0, 0, 0};
        p.ch[0] = {0, 0, 0};
        p.ch[1] = {0, 0, 0};
        if (fields == 9) { sw = 0; fields = 10; }
        if (fields != 10) { err = "config.init: could not read coordinates for particle " + std::to_string(i + 1); return -1; }
        p.switched = sw;
        p.pos.x /= c.box.x; p.pos.y /= c.box.y; p.pos.z /= c.box.z;
        // Cuboid::usePBC(Vector&) (geometry.h:78-97)
        while (p.pos.x < 0.0) p.pos.x += 1.0;
        while (p.pos.x > 1.0) p.pos.x -= 1.0;
        while (p.pos.y < 0.0) p.pos.y += 1.0;
        while (p.pos.y > 1.0) p.pos.y -= 1.0;
        while (p.pos.z < 0.0) p.pos.z += 1.0;
        while (p.pos.z > 1.0) p.pos.z -= 1.0;
        int g = t.ia[p.type][p.type].geotype[0];
        if (g < SP && dot(p.dir, p.dir) < kZEROTOL) { err = "config.init: null direction vector for particle " + std::to_string(i + 1); return -1; }
        normalise(p.dir);
        if (g < SP && g != SCN && dot(p.pd[0], p.pd[0]) < kZEROTOL) { err = "config.init: null patch vector for particle " + std::to_string(i + 1); return -1; }
        orthogonalise(p.pd[0], p.dir);
        normalise(p.pd[0]);
        if (p.switched) {          // the particle carries its switch type (inicializer.cpp:226-236)
            if (p.switchtype < 0) {
                err = "config.init: particle " + std::to_string(i + 1) + " switched even though it has no switchtype";
                return -1;
            }
            std::swap(p.type, p.switchtype);
        }
    }
    // Conf::makeMoleculeWhole for every chain (inicializer.cpp:268-278, Conf.h:373-382)
    for (int m = 0; m < c.molTypeCount; ++m) {
        int size = (int)t.mols[m].types.size();
        if (size <= 1) continue;
        for (int s = c.first[m]; s + size <= c.first[m + 1]; s += size) {
            for (int k = s + 1; k < s + size; ++k) {
                Vec3 r = image(c.p[k].pos, c.p[k - 1].pos, c.box);
                r.x /= c.box.x; r.y /= c.box.y; r.z /= c.box.z;
                c.p[k].pos = {c.p[k - 1].pos.x + r.x, c.p[k - 1].pos.y + r.y, c.p[k - 1].pos.z + r.z};
            }
        }
    }
    return 0;
}

void particleInit(Particle& p, const IaParam& d) {
    int g = d.geotype[0];
    if (g == SCA || g == SCN) return;
    normalise(p.dir);
    orthogonalise(p.pd[0], p.dir);
    normalise(p.pd[0]);
    if (g == PSC || g == CPSC || g == TPSC || g == TCPSC) {
        p.ps[0] = p.pd[0]; rotateAbout(p.ps[0], p.dir, d.pcoshalfi[0], d.psinhalfi[0]);
        p.ps[1] = p.pd[0]; rotateAbout(p.ps[1], p.dir, d.pcoshalfi[0], -1.0 * d.psinhalfi[0]);
    }
    if (isTwoPatch(g)) {
        p.pd[1] = p.pd[0];
        rotateAbout(p.pd[1], p.dir, d.csecpatchrot[0], d.ssecpatchrot[0]);
        orthogonalise(p.pd[1], p.dir);
        normalise(p.pd[1]);
    }
    if (g == TPSC || g == TCPSC) {
        p.ps[2] = p.pd[1]; rotateAbout(p.ps[2], p.dir, d.pcoshalfi[2], d.psinhalfi[2]);
        p.ps[3] = p.pd[1]; rotateAbout(p.ps[3], p.dir, d.pcoshalfi[2], -1.0 * d.psinhalfi[2]);
    }
    if (isChiral(g)) {
        p.ch[0] = p.dir; rotateAbout(p.ch[0], p.pd[0], d.chiral_cos[0], d.chiral_sin[0]);
        p.ps[0] = p.pd[0]; rotateAbout(p.ps[0], p.ch[0], d.pcoshalfi[0], d.psinhalfi[0]);
        p.ps[1] = p.pd[0]; rotateAbout(p.ps[1], p.ch[0], d.pcoshalfi[0], -1.0 * d.psinhalfi[0]);
    }
    if (g == TCHPSC || g == TCHCPSC) {
        p.ch[1] = p.dir; rotateAbout(p.ch[1], p.pd[1], d.chiral_cos[0], d.chiral_sin[0]);
        p.ps[2] = p.pd[1]; rotateAbout(p.ps[2], p.ch[1], d.pcoshalfi[2], d.psinhalfi[2]);
        p.ps[3] = p.pd[1]; rotateAbout(p.ps[3], p.ch[1], d.pcoshalfi[2], -1.0 * d.psinhalfi[2]);
    }
}

void partVecInit(const Topology& t, Config& c) {   // Conf::partVecInit (Conf.cpp:97-102)
    for (auto& p : c.p)
        if (t.ia[p.type][p.type].geotype[0] < SP) particleInit(p, t.ia[p.type][p.type]);
}

std::string drawConfig(const Config& c) {
    std::string out;
    char buf[512];
    std::snprintf(buf, sizeof buf, "%15.8e %15.8e %15.8e\n", c.box.x, c.box.y, c.box.z);
    out += buf;
    for (const Particle& p : c.p) {
        std::snprintf(buf, sizeof buf, "%15.8e %15.8e %15.8e   %15.8e %15.8e %15.8e   %15.8e %15.8e %15.8e %d %d\n",
                      c.box.x * ((p.pos.x) - anInt(p.pos.x)), c.box.y * ((p.pos.y) - anInt(p.pos.y)),
                      c.box.z * ((p.pos.z) - anInt(p.pos.z)), p.dir.x, p.dir.y, p.dir.z, p.pd[0].x, p.pd[0].y,
                      p.pd[0].z, p.switched, p.molType);
        out += buf;
    }
    return out;
}

}  // namespace scg
