// Host side of a mechanism: validation, canonical constants, transport fits and packed tables.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/combustion_gb300.h"

namespace cbg {

struct Work {
    double flops = 0, exps = 0, logs = 0, divs = 0, sqrts = 0, bytes_in = 0, bytes_out = 0;
};

struct HostMechanism {
    int K = 0, R = 0, A = 0;
    int n_eff = 0;  // reactions with third-body efficiencies (three-body and falloff)
    std::vector<double> W, split, nasa7;  // [K], [K], [K*14]
    std::vector<int32_t> geometry;
    std::vector<double> diameter, well_depth, polarizability, dipole, rot, dof;
    std::vector<uint8_t> reactants, products;  // [R*K]
    std::vector<int32_t> model;
    std::vector<double> rate, k0, troe, sri, eff;  // [R*3], [R*3], [R*4], [R*5], [R*K]

    std::vector<uint8_t> rates_blob;
    std::vector<uint8_t> rates_mixed_blob;  // tables of the mixed-precision form
    Work rates_work;

    bool transport_ready = false;
    double T0 = 0, mu0 = 0, lambda0 = 0;
    std::vector<double> fit_cond, fit_visc, fit_diff;  // raw fits [K*5], [K*5], [K*K*5]
    std::vector<uint8_t> transport_blob;
    std::vector<uint8_t> transport_mixed_blob;
    Work transport_work;
};

// Copies and validates the description, finds the active species and packs the rates tables.
// Returns CB_OK or an error code with a message.
int build_mechanism(const cb_mech_desc* d, HostMechanism& m, std::string& err);
// Fits the species properties and packs the transport tables for the given normalisation.
int build_transport(HostMechanism& m, double T0, double mu0, double lambda0, std::string& err);

struct MathTables;
MathTables make_math_tables();

// Transport physics of one species or pair at temperature T (SI), used by the fits.
double species_viscosity(const HostMechanism& m, int k, double T);
double species_conductivity(const HostMechanism& m, int k, double T);
double pair_diffusivity(const HostMechanism& m, int a, int b, double T);

}  // namespace cbg
