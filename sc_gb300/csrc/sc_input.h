// sc_input.h -- the reference's input surface: options, top.init, config.init.
//
// Host-side C++ that reads the three files the reference reads and derives the
// same interaction table and particle vectors.  Semantics follow
//   Sim::readOptions            scOOP/structures/sim.h:123-406
//   Inicializer::readTopoFile   scOOP/mc/inicializer.cpp:453-585 (fillTypes 660-852, fillMol 929-1108)
//   Inicializer::initConfig     scOOP/mc/inicializer.cpp:89-298
//   Topo::genParamPairs / genTopoParams  scOOP/structures/topo.cpp:5-153
//   Particle::init              scOOP/structures/particle.cpp:3-79
// Errors are reported as return codes with a message, never by exiting.
#pragma once

#include <string>
#include <vector>

#include "sc_common.h"

namespace scg {

struct Vec3 { double x = 0, y = 0, z = 0; };

struct Particle {
    Vec3 pos, dir, pd[2], ps[4], ch[2];
    int type = 0, molType = 0, switchtype = -1, switched = 0;   // switchtype: the other type (-1: none)
};

// Full Ia_param (scOOP/structures/structures.h:187-254).
struct IaParam {
    int geotype[2] = {0, 0};
    double sigma = 0, sigmaSq = 0, epsilon = 0, A = 0, B = 0, pdis = 0, pdisSq = 0, pswitch = 0, pswitchINV = 0;
    double pangl[4] = {0, 0, 0, 0}, panglsw[4] = {0, 0, 0, 0}, pcangl[4] = {0, 0, 0, 0}, pcanglsw[4] = {0, 0, 0, 0};
    double rcut = 0, rcutSq = 0, rcutwca = 0, rcutwcaSq = 0;
    double pcoshalfi[4] = {0, 0, 0, 0}, psinhalfi[4] = {0, 0, 0, 0};
    double csecpatchrot[2] = {0, 0}, ssecpatchrot[2] = {0, 0};
    double volume = 0, pvolscale = 0;
    double len[2] = {0, 0}, half_len[2] = {0, 0}, chiral_cos[2] = {0, 0}, chiral_sin[2] = {0, 0};
    double parallel = 0;
    bool exclude = false;
};

struct MolType {
    std::string name;
    std::vector<int> types;
    std::vector<int> switchTypes;      // per particle of the molecule: its switch type, -1 for none
    std::vector<double> deltaMu;       // per particle: the chemical-potential difference of the switch
    double bond1eq = -1, bond1c = -1, bond2eq = -1, bond2c = -1, bonddeq = -1, bonddc = -1, bondheq = -1, bondhc = -1;
    double angle1eq = -1, angle1c = -1, angle2eq = -1, angle2c = -1;
    double activity = -1;
};

// Values of the options file after the unit conversions of sim.h:359-381.
struct Options {
    long write_cluster = 0, adjust = 0, movie = 0, nequil = 0, nsweeps = 0, nrepchange = 0, nGrandCanon = 0,
         nClustMove = 0, paramfrq = 0, report = 0, seed = 0;
    int pairlist_update = 0, ptype = 0, wlm[2] = {0, 0}, wlmtype = 0;
    double press = 0, paralpress = 0, edge_mx = 0, shave = 0, chainprob = 0, switchprob = 0, temper = 0,
           paraltemper = 0, transmx = 0, rotmx_deg = 0, coneAngle = 0, chainmmx = 0, chainrmx_deg = 0;
    double rot_angle = 0;      // rotmx/180*PIH*0.5, the half-angle bound of pscRotate
    double chain_angle = 0;    // chainrmx/180*PIH
    double trans_type[MAXT];   // per-type displacement length (transmx, or transmx_type entries)
};

struct Topology {
    IaParam ia[MAXT][MAXT];
    bool exclusions[MAXT][MAXT] = {};
    std::vector<MolType> mols;
    std::vector<std::pair<std::string, long>> system;
    double sqmaxcut = 0, maxcut = 0;
};

struct Config {
    Vec3 box{0, 0, 0};
    std::vector<Particle> p;
    std::vector<int> first;    // ParticleVector::first, size molTypeCount+1
    int molTypeCount = 0;
};

int readOptionsText(const std::string& text, Options& o, std::string& err);
int readTopologyText(const std::string& text, Topology& t, std::string& err);
// Builds the particle list from [System] (Inicializer::setParticlesParamss) and ParticleVector::first.
int buildParticles(const Topology& t, Config& c, std::string& err);
int readConfigText(const std::string& text, const Topology& t, Config& c, std::string& err);
void particleInit(Particle& p, const IaParam& diag);
void partVecInit(const Topology& t, Config& c);
std::string drawConfig(const Config& c);   // Conf::draw (scOOP/structures/Conf.h:388-425), config.last format

Vec3 image(const Vec3& r1, const Vec3& r2, const Vec3& box);
double anInt(double d);

}  // namespace scg
