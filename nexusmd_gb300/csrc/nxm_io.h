// Host-side inputs and outputs of the Simulate path: the system/state XML
// readers and the three report files, in the reference's formats.
#pragma once

#include <string>
#include <vector>

namespace nxm {

// SystemXMLParser.h:10-39 (PTorsionParams, BondParams, AngleParams,
// NonbondedParticle, NonbondedException, NonbondedParams)
struct TorsionP {
    int p1, p2, p3, p4;
    double k, phase;
    int periodicity;
};
struct BondP {
    int p1, p2;
    double d, k;
};
struct AngleP {
    int p1, p2, p3;
    double a, k;
};
struct NbParticle {
    double q, sig, eps;
};
struct NbException {
    int p1, p2;
    double q, sig, eps;
};
struct NbParams {
    double alpha = 0, cutoff = 0, ewaldTolerance = 0, rfDielectric = 0, switchingDistance = 0;
    int dispersionCorrection = 0, exceptionsUsePeriodic = 0, forceGroup = 0, includeDirectSpace = 0, ljAlpha = 0,
        ljnx = 0, ljny = 0, ljnz = 0, method = 0, nx = 0, ny = 0, nz = 0, recipForceGroup = 0,
        useSwitchingFunction = 0, version = 0;
    std::vector<NbParticle> particles;
    std::vector<NbException> exceptions;
};

struct ParsedSystem {
    std::vector<double> masses;
    std::vector<TorsionP> torsions;
    std::vector<BondP> bonds;
    std::vector<AngleP> angles;
    NbParams nb;
    std::vector<double> positions;   // [n][3] from the state file
    std::vector<double> velocities;  // [n][3] <Velocities> of the state file, when it has them
};

// printf("%*.*f", width, prec, x) without the C library's general
// conversion: for finite |x| < 2^40 and prec <= 17 the double's exact value
// m * 2^-s is scaled by 10^prec in 128-bit integers and rounded half to
// even (what glibc prints under the default rounding mode), the sign of
// negative values and of negative zero kept; anything else goes through
// snprintf.  `out` must hold kFixedCharsMax bytes; returns the length.
constexpr int kFixedCharsMax = 400;
int fixed_chars(double x, int prec, int width, char *out);

// A checkpoint in OpenMM's state format: <PeriodicBoxVectors> (orthorhombic
// edges), <Positions> and <Velocities>, every value printed with 17
// significant digits so that reading it back gives the same doubles.
bool write_state_xml(const std::string &path, int n, const double *xyz, const double *vel, const double box[3],
                     long long step, double time_ps);

// Each parser mirrors one SystemXMLParser / StateXMLParser function: on a
// file that does not parse it prints the reference's message to stderr and
// returns an empty result.
std::vector<double> parse_masses(const std::string &system_xml);
std::vector<TorsionP> parse_torsions(const std::string &system_xml);
std::vector<BondP> parse_bonds(const std::string &system_xml);
std::vector<AngleP> parse_angles(const std::string &system_xml);
NbParams parse_nonbonded(const std::string &system_xml);
std::vector<double> parse_state_positions(const std::string &state_xml);
// All of the above from one read of each file (the reference reads the
// system file five times).
ParsedSystem parse_all(const std::string &system_xml, const std::string &state_xml);
// Whether a file parses as XML (no message).
bool xml_ok(const std::string &path);

// One PDB ATOM record as the reporter keeps it (Reporter.h:10-21).
struct PdbAtom {
    int atomNum = 0;
    std::string atomName, resName;
    char chainID = 'A';
    int resSeq = 0;
    double coords[3] = {0, 0, 0};
    double occupancy = 0, tempFactor = 0;
    std::string element, recordType;
};

// The three report files of Reporter.cpp, written with the same bytes.
class ReportWriter {
public:
    ReportWriter(const std::string &input_pdb, const std::string &output_pdb);
    // Reporter::pdbOutputGeneratorPart1: template from the input PDB, then
    // the REMARK and CRYST1 lines (file truncated).
    bool pdb_part1();
    // Reporter::pdbOutputGeneratorPart2: one MODEL with positions x10 (nm -> A);
    // `announce` prints the model number to stdout as the reference does
    // (a caller that reports from another thread prints it itself, in order).
    bool pdb_part2(const double *pos, int model, bool announce = true);
    // Reporter::TotalEnergyReport: header and fixed 10-digit numbers on the
    // step-0 open only, default stream formatting afterwards.
    bool total_energy(double ke, double pe, double te, int step);
    // Reporter::TestPVFReport.  The lines are formatted by `threads` threads
    // over contiguous atom ranges and written in order: the same bytes for
    // any thread count.
    bool pvf(const double *pos, const double *vel, const double *frc, int n, int step, int threads = 1);
    const std::string &error() const { return err_; }

private:
    std::string in_, out_, pbc_line_, err_;
    std::vector<PdbAtom> tmpl_;
    std::vector<std::string> pre_, post_;  // each ATOM record's text around its coordinates
};

}  // namespace nxm
