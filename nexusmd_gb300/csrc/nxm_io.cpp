// System/state XML readers (core/common/src/SystemXMLParser.cpp:18-196,
// StateXMLParser.cpp:17-37) and the report writers (core/baseline/src/
// Reporter.cpp:26-229), producing the same values and the same file bytes.
#include "nxm_io.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <iostream>
#include <set>
#include <sstream>
#include <thread>

#include "nxm_xml.h"

namespace nxm {

namespace {

bool load(const std::string &path, XmlDoc &doc) {
    doc = xml_load_file(path);
    if (!doc.error.empty()) {
        std::cerr << "XML [" << path << "] parsed with errors, Error description: " << doc.error << "\n";
        return false;
    }
    return true;
}

const XmlNode *forces_of(const XmlDoc &d) {
    const XmlNode *sys = d.root.child("System");
    return sys ? sys->child("Forces") : nullptr;
}

std::vector<double> masses_of(const XmlDoc &d) {
    std::vector<double> m;
    const XmlNode *sys = d.root.child("System");
    const XmlNode *parts = sys ? sys->child("Particles") : nullptr;
    if (parts)
        for (auto *p : parts->children_named("Particle")) m.push_back(p->as_double("mass"));
    return m;
}

template <typename F>
void each_force(const XmlDoc &d, const char *type, F fn) {
    const XmlNode *fs = forces_of(d);
    if (!fs) return;
    for (auto *f : fs->children_named("Force")) {
        const char *t = f->attr("type");
        if (t && std::string(t) == type) fn(f);
    }
}

std::vector<TorsionP> torsions_of(const XmlDoc &d) {
    std::vector<TorsionP> out;
    each_force(d, "PeriodicTorsionForce", [&](const XmlNode *f) {
        const XmlNode *ts = f->child("Torsions");
        if (!ts) return;
        for (auto *t : ts->children_named("Torsion"))
            out.push_back(TorsionP{t->as_int("p1"), t->as_int("p2"), t->as_int("p3"), t->as_int("p4"),
                                   t->as_double("k"), t->as_double("phase"), t->as_int("periodicity")});
    });
    return out;
}

std::vector<BondP> bonds_of(const XmlDoc &d) {
    std::vector<BondP> out;
    each_force(d, "HarmonicBondForce", [&](const XmlNode *f) {
        const XmlNode *bs = f->child("Bonds");
        if (!bs) return;
        for (auto *b : bs->children_named("Bond"))
            out.push_back(BondP{b->as_int("p1"), b->as_int("p2"), b->as_double("d"), b->as_double("k")});
    });
    return out;
}

std::vector<AngleP> angles_of(const XmlDoc &d) {
    std::vector<AngleP> out;
    each_force(d, "HarmonicAngleForce", [&](const XmlNode *f) {
        const XmlNode *as = f->child("Angles");
        if (!as) return;
        for (auto *a : as->children_named("Angle"))
            out.push_back(AngleP{a->as_int("p1"), a->as_int("p2"), a->as_int("p3"), a->as_double("a"), a->as_double("k")});
    });
    return out;
}

NbParams nonbonded_of(const XmlDoc &d) {
    NbParams p;
    const XmlNode *fs = forces_of(d);
    if (!fs) {
        std::cerr << "No Forces node found in the XML.\n";
        return p;
    }
    const XmlNode *f = nullptr;
    for (auto *c : fs->children_named("Force")) {
        const char *t = c->attr("type");
        if (t && std::string(t) == "NonbondedForce") {
            f = c;
            break;
        }
    }
    if (!f) {
        std::cerr << "No NonbondedForce found in the XML.\n";
        return p;
    }
    p.alpha = f->as_double("alpha");
    p.cutoff = f->as_double("cutoff");
    p.dispersionCorrection = f->as_int("dispersionCorrection");
    p.ewaldTolerance = f->as_double("ewaldTolerance");
    p.exceptionsUsePeriodic = f->as_int("exceptionsUsePeriodic");
    p.forceGroup = f->as_int("forceGroup");
    p.includeDirectSpace = f->as_int("includeDirectSpace");
    p.ljAlpha = f->as_int("ljAlpha");
    p.ljnx = f->as_int("ljnx");
    p.ljny = f->as_int("ljny");
    p.ljnz = f->as_int("ljnz");
    p.method = f->as_int("method");
    p.nx = f->as_int("nx");
    p.ny = f->as_int("ny");
    p.nz = f->as_int("nz");
    p.recipForceGroup = f->as_int("recipForceGroup");
    p.rfDielectric = f->as_double("rfDielectric");
    p.switchingDistance = f->as_double("switchingDistance");
    p.useSwitchingFunction = f->as_int("useSwitchingFunction");
    p.version = f->as_int("version");
    if (const XmlNode *ps = f->child("Particles"))
        for (auto *q : ps->children_named("Particle"))
            p.particles.push_back(NbParticle{q->as_double("q"), q->as_double("sig"), q->as_double("eps")});
    if (const XmlNode *es = f->child("Exceptions"))
        for (auto *e : es->children_named("Exception"))
            p.exceptions.push_back(NbException{e->as_int("p1"), e->as_int("p2"), e->as_double("q"), e->as_double("sig"),
                                               e->as_double("eps")});
    return p;
}

// <State><Positions><Position x y z/> (StateXMLParser.cpp:17-37), and the
// same for <Velocities><Velocity/>, which OpenMM writes beside them and the
// reference does not read.
std::vector<double> vectors_of(const XmlDoc &d, const char *group, const char *item) {
    std::vector<double> out;
    const XmlNode *st = d.root.child("State");
    const XmlNode *ps = st ? st->child(group) : nullptr;
    if (ps)
        for (auto *q : ps->children_named(item)) {
            out.push_back(q->as_double("x"));
            out.push_back(q->as_double("y"));
            out.push_back(q->as_double("z"));
        }
    return out;
}

std::vector<double> positions_of(const XmlDoc &d) { return vectors_of(d, "Positions", "Position"); }

}  // namespace

std::vector<double> parse_masses(const std::string &f) {
    XmlDoc d;
    return load(f, d) ? masses_of(d) : std::vector<double>();
}
std::vector<TorsionP> parse_torsions(const std::string &f) {
    XmlDoc d;
    return load(f, d) ? torsions_of(d) : std::vector<TorsionP>();
}
std::vector<BondP> parse_bonds(const std::string &f) {
    XmlDoc d;
    return load(f, d) ? bonds_of(d) : std::vector<BondP>();
}
std::vector<AngleP> parse_angles(const std::string &f) {
    XmlDoc d;
    return load(f, d) ? angles_of(d) : std::vector<AngleP>();
}
NbParams parse_nonbonded(const std::string &f) {
    XmlDoc d;
    return load(f, d) ? nonbonded_of(d) : NbParams();
}
std::vector<double> parse_state_positions(const std::string &f) {
    XmlDoc d;
    return load(f, d) ? positions_of(d) : std::vector<double>();
}

bool xml_ok(const std::string &path) { return xml_load_file(path).error.empty(); }

ParsedSystem parse_all(const std::string &system_xml, const std::string &state_xml) {
    ParsedSystem ps;
    XmlDoc st;
    if (!state_xml.empty() && load(state_xml, st)) {
        ps.positions = positions_of(st);
        ps.velocities = vectors_of(st, "Velocities", "Velocity");
    }
    XmlDoc d;
    if (!system_xml.empty() && load(system_xml, d)) {
        ps.masses = masses_of(d);
        ps.torsions = torsions_of(d);
        ps.bonds = bonds_of(d);
        ps.angles = angles_of(d);
        ps.nb = nonbonded_of(d);
    }
    return ps;
}

// ------------------------------------------------------------------ reports

namespace {
const char kDigitPairs[201] =
    "00010203040506070809101112131415161718192021222324252627282930313233343536373839"
    "40414243444546474849505152535455565758596061626364656667686970717273747576777879"
    "8081828384858687888990919293949596979899";
}  // namespace

int fixed_chars(double x, int prec, int width, char *out) {
    static const unsigned long long p10[18] = {1ULL,
                                               10ULL,
                                               100ULL,
                                               1000ULL,
                                               10000ULL,
                                               100000ULL,
                                               1000000ULL,
                                               10000000ULL,
                                               100000000ULL,
                                               1000000000ULL,
                                               10000000000ULL,
                                               100000000000ULL,
                                               1000000000000ULL,
                                               10000000000000ULL,
                                               100000000000000ULL,
                                               1000000000000000ULL,
                                               10000000000000000ULL,
                                               100000000000000000ULL};
    if (!(std::fabs(x) < 1099511627776.0) || prec < 0 || prec > 17 || width > 64)
        return std::min(std::snprintf(out, kFixedCharsMax, "%*.*f", width, prec, x), kFixedCharsMax - 1);
    const bool neg = std::signbit(x);
    // integer part and fraction, both exact: |x| < 2^40, so ip fits and
    // |x| - ip is representable
    const double ax = std::fabs(x);
    unsigned long long ip = (unsigned long long)ax;
    const double fr = ax - (double)ip;
    // the fraction's exact value m * 2^-s scaled by 10^prec, rounded half to
    // even on the whole number ip * 10^prec + fp (10^prec is even for prec > 0)
    unsigned long long bits;
    std::memcpy(&bits, &fr, sizeof bits);
    const int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long m = bits & ((1ULL << 52) - 1);
    int s;
    if (ex == 0) {
        s = 1074;
    } else {
        m |= 1ULL << 52;
        s = 1075 - ex;  // >= 53: fr < 1
    }
    using u128 = unsigned __int128;
    const u128 P = (u128)m * p10[prec];  // < 2^110
    unsigned long long fp = 0;
    if (s < 128) {
        const u128 q = P >> s;
        const u128 rem = P - (q << s), half = (u128)1 << (s - 1);
        fp = (unsigned long long)q;
        const unsigned long long par = prec > 0 ? fp : fp + ip;
        if (rem > half || (rem == half && (par & 1))) ++fp;
        if (fp == p10[prec]) {  // rounded up to the next integer
            fp = 0;
            ++ip;
        }
    }  // else the fraction is below half an ulp of the last place: zero
    // digits right to left into tmp[..64): the fraction as exactly prec
    // digits, then the integer part; two digits per step, in 32-bit pieces
    char tmp[64];
    char *e = tmp + 64, *p = e;
    auto put8 = [&](unsigned v, int nd) {  // nd <= 8 digits of v (v < 10^nd)
        for (; nd >= 2; nd -= 2) {
            p -= 2;
            std::memcpy(p, kDigitPairs + 2 * (v % 100), 2);
            v /= 100;
        }
        if (nd) *--p = (char)('0' + v);
    };
    if (prec > 0) {
        int nd = prec;
        while (nd > 8) {
            put8((unsigned)(fp % 100000000ULL), 8);
            fp /= 100000000ULL;
            nd -= 8;
        }
        put8((unsigned)fp, nd);
        *--p = '.';
    }
    while (ip >= 100000000ULL) {
        put8((unsigned)(ip % 100000000ULL), 8);
        ip /= 100000000ULL;
    }
    {
        unsigned v = (unsigned)ip;
        do {
            *--p = (char)('0' + v % 10);
            v /= 10;
        } while (v);
    }
    if (neg) *--p = '-';
    const int t = (int)(e - p);
    int len = 0;
    for (int pad = width - t; pad > 0; --pad) out[len++] = ' ';
    std::memcpy(out + len, p, t);
    len += t;
    out[len] = 0;
    return len;
}

namespace {

// "%d" of a non-negative int
int uint_chars(int v, char *out) {
    char tmp[16];
    int t = 0;
    do {
        tmp[t++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    int len = 0;
    while (t) out[len++] = tmp[--t];
    return len;
}

const std::set<std::string> kAminoAcids = {"ALA", "ARG", "ASN", "ASP", "CYS", "GLN", "GLU", "GLY", "HIS", "ILE",
                                           "LEU", "LYS", "MET", "PHE", "PRO", "SER", "THR", "TRP", "TYR", "VAL"};

// Reporter.cpp:98-107
std::string element_of(const std::string &name) {
    if (name.empty()) return "";
    std::string e(1, name[0]);
    if (name.size() > 1 && std::islower((unsigned char)name[1])) e += name[1];
    return e;
}

// Reporter.cpp:109-118: whitespace-separated fields, chain fixed to 'A';
// a field that does not read leaves the rest at zero.
PdbAtom parse_pdb_line(const std::string &line) {
    PdbAtom a;
    std::istringstream ss(line);
    ss >> a.recordType >> a.atomNum >> a.atomName >> a.resName >> a.resSeq >> a.coords[0] >> a.coords[1] >> a.coords[2] >>
        a.occupancy >> a.tempFactor;
    a.chainID = 'A';
    a.element = element_of(a.atomName);
    a.recordType = kAminoAcids.count(a.resName) ? "ATOM  " : "HETATM";
    return a;
}

std::string date_today() {
    std::time_t t = std::time(nullptr);
    char buf[32];
    std::strftime(buf, sizeof buf, "%Y-%m-%d", std::localtime(&t));
    return buf;
}

// Reporter.cpp:145-169
std::string pdb_line(const PdbAtom &a) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "%-6s%5d %-4s %3s %c%4d    %8.3f%8.3f%8.3f%6.2f%6.2f          %-2s",
                  a.recordType.c_str(), a.atomNum, a.atomName.c_str(), a.resName.c_str(), a.chainID, a.resSeq,
                  a.coords[0], a.coords[1], a.coords[2], a.occupancy, a.tempFactor, a.element.c_str());
    return buf;
}

}  // namespace

ReportWriter::ReportWriter(const std::string &input_pdb, const std::string &output_pdb)
    : in_(input_pdb), out_(output_pdb) {}

bool ReportWriter::pdb_part1() {
    std::ofstream out(out_);
    std::ifstream in(in_);
    if (!in) {
        std::cerr << "Failed to open input file." << std::endl;
    } else {
        std::string line;
        while (std::getline(in, line)) {
            if (line.substr(0, 4) == "ATOM")
                tmpl_.push_back(parse_pdb_line(line));
            else if (line.substr(0, 6) == "CRYST1")
                pbc_line_ = line;
        }
    }
    out << "REMARK   Generated by Nexaus 1.0.0, " << date_today() << std::endl;
    out << pbc_line_ << std::endl;
    return true;
}

bool ReportWriter::pdb_part2(const double *pos, int model, bool announce) {
    std::ofstream out(out_, std::ios::out | std::ios::app);
    if (!out.is_open()) {
        std::cerr << "Unable to open the file: " << out_ << std::endl;
        return false;
    }
    if (announce) std::cout << model << "   ";
    // the record's text before and after the coordinates is fixed per atom
    if (pre_.size() != tmpl_.size()) {
        pre_.clear();
        post_.clear();
        char buf[256];
        for (const PdbAtom &a : tmpl_) {
            std::snprintf(buf, sizeof buf, "%-6s%5d %-4s %3s %c%4d    ", a.recordType.c_str(), a.atomNum,
                          a.atomName.c_str(), a.resName.c_str(), a.chainID, a.resSeq);
            pre_.push_back(buf);
            std::snprintf(buf, sizeof buf, "%6.2f%6.2f          %-2s", a.occupancy, a.tempFactor, a.element.c_str());
            post_.push_back(buf);
        }
    }
    std::string text = "MODEL        " + std::to_string(model) + "\n";
    text.reserve(tmpl_.size() * 82 + 64);
    std::vector<char> line(pre_.empty() ? 1 : 600 + 3 * kFixedCharsMax);
    for (size_t i = 0; i < tmpl_.size(); ++i) {
        PdbAtom a = tmpl_[i];
        for (int c = 0; c < 3; ++c) a.coords[c] = pos[3 * (size_t)(a.atomNum - 1) + c] * 10.0;
        size_t k = 0;
        if (pre_[i].size() + post_[i].size() < 256) {
            std::memcpy(line.data(), pre_[i].data(), pre_[i].size());
            k = pre_[i].size();
            for (int c = 0; c < 3; ++c) k += fixed_chars(a.coords[c], 3, 8, line.data() + k);
            std::memcpy(line.data() + k, post_[i].data(), post_[i].size());
            k += post_[i].size();
        }
        if (k > 0 && k < 256) {
            text.append(line.data(), k);
        } else {
            text += pdb_line(a);  // the reference's 256-byte line buffer truncates: as it does
        }
        text += '\n';
        if (i == tmpl_.size() - 1) {
            char buf[128];
            std::snprintf(buf, sizeof buf, "%-6s%5d %-4s %3s %c%4d", "TER", tmpl_[i].atomNum + 1, "",
                          tmpl_[i].resName.c_str(), tmpl_[i].chainID, tmpl_[i].resSeq);
            text += buf;
            text += '\n';
        }
    }
    text += "ENDMDL\n";
    out << text;
    out.flush();
    return true;
}

bool ReportWriter::total_energy(double ke, double pe, double te, int step) {
    std::string name = "TotalEnergy" + out_;
    std::ofstream out(name, step == 0 ? std::ios::out : (std::ios::out | std::ios::app));
    if (!out.is_open()) {
        std::cerr << "Unable to open the file: " << name << std::endl;
        return false;
    }
    char buf[256];
    if (step == 0) {
        out << "Step\tTotal Kinetic Energy (kJ/mol)\tTotal Potential Energy (kJ/mol)\tTotal Energy (kJ/mol)\n";
        std::snprintf(buf, sizeof buf, "%5d%25.10f%30.10f%25.10f\n", step, ke, pe, te);
    } else {
        std::snprintf(buf, sizeof buf, "%5d%25g%30g%25g\n", step, ke, pe, te);
    }
    out << buf;
    return true;
}

bool ReportWriter::pvf(const double *pos, const double *vel, const double *frc, int n, int step, int threads) {
    std::string name = "PVFReport" + out_;
    std::ofstream out(name, step == 0 ? std::ios::out : (std::ios::out | std::ios::app));
    if (!out.is_open()) {
        std::cerr << "Unable to open the file: " << name << std::endl;
        return false;
    }
    out << "Step" << step << "\n";
    out << "ID\tPosition(nm)\t\t\tVelocity(nm / ps)\t\tForce(kJ / mol * nm)\n";
    // "%d\t(%10.10f, %10.10f, %10.10f)\t(...)\t(...)\n" per atom
    auto format = [&](int i0, int i1, std::string &buf) {
        buf.reserve((size_t)(i1 - i0) * 160);
        char line[16 + 9 * (kFixedCharsMax + 2) + 16];
        for (int i = i0; i < i1; ++i) {
            const double *col[3] = {pos + 3 * (size_t)i, vel + 3 * (size_t)i, frc + 3 * (size_t)i};
            int k = uint_chars(i + 1, line);
            line[k++] = '\t';
            for (int g = 0; g < 3; ++g) {
                line[k++] = '(';
                for (int c = 0; c < 3; ++c) {
                    k += fixed_chars(col[g][c], 10, 10, line + k);
                    if (c < 2) {
                        line[k++] = ',';
                        line[k++] = ' ';
                    }
                }
                line[k++] = ')';
                line[k++] = g < 2 ? '\t' : '\n';
            }
            buf.append(line, k);
        }
    };
    int nt = std::max(1, std::min(threads, n / 1024 + 1));
    std::vector<std::string> parts(nt);
    if (nt == 1) {
        format(0, n, parts[0]);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back(format, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt), std::ref(parts[t]));
        for (auto &th : pool) th.join();
    }
    for (auto &p : parts) out << p;
    out << "\n";
    return true;
}

bool write_state_xml(const std::string &path, int n, const double *xyz, const double *vel, const double box[3],
                     long long step, double time_ps) {
    std::ofstream out(path);
    if (!out.is_open()) {
        std::cerr << "Unable to open the file: " << path << std::endl;
        return false;
    }
    std::string buf;
    buf.reserve((size_t)n * 160 + 512);
    char line[256];
    std::snprintf(line, sizeof line,
                  "<?xml version=\"1.0\" ?>\n<State stepCount=\"%lld\" time=\"%.17g\" type=\"State\" version=\"1\">\n",
                  step, time_ps);
    buf += line;
    std::snprintf(line, sizeof line,
                  "\t<PeriodicBoxVectors>\n\t\t<A x=\"%.17g\" y=\"0\" z=\"0\"/>\n\t\t<B x=\"0\" y=\"%.17g\" z=\"0\"/>\n"
                  "\t\t<C x=\"0\" y=\"0\" z=\"%.17g\"/>\n\t</PeriodicBoxVectors>\n",
                  box[0], box[1], box[2]);
    buf += line;
    const double *arr[2] = {xyz, vel};
    const char *group[2] = {"Positions", "Velocities"}, *item[2] = {"Position", "Velocity"};
    for (int k = 0; k < 2; ++k) {
        if (!arr[k]) continue;
        buf += std::string("\t<") + group[k] + ">\n";
        for (int i = 0; i < n; ++i) {
            const double *p = arr[k] + 3 * (size_t)i;
            std::snprintf(line, sizeof line, "\t\t<%s x=\"%.17g\" y=\"%.17g\" z=\"%.17g\"/>\n", item[k], p[0], p[1], p[2]);
            buf += line;
        }
        buf += std::string("\t</") + group[k] + ">\n";
    }
    buf += "</State>\n";
    out << buf;
    return (bool)out;
}

}  // namespace nxm
