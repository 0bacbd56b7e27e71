// oracle/mdref.cpp -- CPU FP64 restatement of the moldyn solver path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU engine is
// checked against.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
// leg of bench.py load it; the product library (libmdgb) never links or
// calls it.
//
// Parity is pinned: tests/test_oracle_golden.py checks every value below
// against the golden numbers in the reference's own unit tests
// (solver/src/lib.rs:77-427, cli/src/tests.rs:35-98), extracted verbatim into
// tests/golden/reference_kats.json by tests/golden/extract_kats.py.
//
// The reference is Rust (no Rust toolchain here), so this is a restatement,
// operation for operation, of:
//   solver/src/solver/potential.rs:27-75     Potential::new_lennard_jones / get_potential_and_force
//   solver/src/solver/potential.rs:141-154   PotentialsDatabase::set_potential / get_potential
//   solver/src/solver/potential.rs:158-216   update_force (O(N^2), rayon over i)
//   solver/src/solver/integrator.rs:14-59    Integrator::VerletMethod::calculate
//   solver/src/initializer/thermostat.rs:24-72  Berendsen / Nose-Hoover
//   solver/src/initializer/barostat.rs:21-49    Berendsen barostat
//   solver/src/macro_parameters/*.rs         COM velocity, energies, pressure, temperature
//   core/src/particle.rs:120-141             State::apply_boundary_conditions
//   core/src/lib.rs:15                       K_B
//   solver/src/initializer/position.rs:25-99 U / FCC lattice fill order
//
// Floating point: every expression keeps the reference's operation order and
// is compiled with -ffp-contract=off (Rust never fuses a*b+c).  Third-party
// arithmetic the reference relies on:
//   nalgebra 0.32  Vector3::norm() = sqrt((x*x + y*y) + z*z); `r / r_abs * f`
//                  is a component-wise divide then multiply; Vector4 `.sum()`
//                  folds component-wise from zero in iteration order.
//   num-traits     `f64.pow(6)` -> powi(6) -> s2 = s*s, s4 = s2*s2, s6 = s2*s4
//                  (binary powering; every ordering of these products yields
//                  the same bits).
//   rayon          only distributes rows i; the j-sum of each row is serial, so
//                  results do not depend on the thread count.
//
// State layout: the reference keeps `Vec<Vec<Particle>>` grouped by type id.
// Here a state is a flat type-major array (all atoms of type 0, then type 1,
// ...) described by `counts[t]`; atom k of type t sits at index
// sum(counts[0..t]) + k, exactly the order `StateToSave::from` flattens to.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// core/src/lib.rs:15
const double OREF_K_B = 1.380648528;

// Potential table entry: {sigma, eps, r_cut, u_cut}
struct oref_lj { double sigma, eps, r_cut, u_cut; };

// solver/src/solver/potential.rs:57-75 get_potential_and_force
static inline void lj_eval(const oref_lj& p, double r, double* u, double* dudr) {
    if (r > p.r_cut) { *u = 0.0; *dudr = 0.0; return; }
    double s = p.sigma / r;
    double s2 = s * s;
    double s4 = s2 * s2;
    double s6 = s2 * s4;
    double s12 = s6 * s6;
    *u = 4.0 * p.eps * (s12 - s6) - p.u_cut;
    *dudr = (24.0 * p.eps / r) * (s6 - 2.0 * s12);
}

// solver/src/solver/potential.rs:27-55 new_lennard_jones: r_cut = 2.5 sigma,
// u_cut = U(r_cut) evaluated with u_cut = 0.
void oref_lj_new(double sigma, double eps, double out[4]) {
    oref_lj p{sigma, eps, sigma * 2.5, 0.0};
    double u, f;
    lj_eval(p, p.r_cut, &u, &f);
    out[0] = sigma; out[1] = eps; out[2] = p.r_cut; out[3] = u;
}

void oref_lj_eval(const double pot[4], double r, double* u, double* dudr) {
    oref_lj p{pot[0], pot[1], pot[2], pot[3]};
    lj_eval(p, r, u, dudr);
}

// Table lookup: pot_table[(t0*ntypes + t1)*4 ...], symmetric, filled by the
// caller from PotentialsDatabase::get_potential (potential.rs:147-154).
static inline oref_lj table_get(const double* table, int ntypes, int a, int b) {
    if (a > b) std::swap(a, b);
    const double* q = table + ((size_t)a * ntypes + b) * 4;
    return oref_lj{q[0], q[1], q[2], q[3]};
}

// solver/src/solver/potential.rs:158-216 update_force.
// Rows [row_begin, row_end) of the flat array are evaluated (row_end < 0 means
// all rows); the bounded-sample CPU baseline times a subset of rows.
int oref_update_force(int ntypes, const int64_t* counts, const double* pos,
                      const double box[3], const double* pot_table,
                      double* force, double* potential, double* temp,
                      int nthreads, int64_t row_begin, int64_t row_end) {
    std::vector<int64_t> off(ntypes + 1, 0);
    for (int t = 0; t < ntypes; ++t) off[t + 1] = off[t] + counts[t];
    const int64_t n = off[ntypes];
    if (row_end < 0 || row_end > n) row_end = n;
    if (row_begin < 0) row_begin = 0;
    // potential.rs:161-169: zero force, potential, temp
    for (int64_t i = row_begin; i < row_end; ++i) {
        force[3 * i] = force[3 * i + 1] = force[3 * i + 2] = 0.0;
        potential[i] = 0.0; temp[i] = 0.0;
    }
    const double bx = box[0], by = box[1], bz = box[2];
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    // potential.rs:171-177: for t1, for t2 >= t1, par over i in t1, serial j in t2
    for (int t1 = 0; t1 < ntypes; ++t1) {
        for (int t2 = t1; t2 < ntypes; ++t2) {
            const oref_lj pot = table_get(pot_table, ntypes, t1, t2);
            const double r_cut = pot.r_cut;
            int64_t ib = std::max(off[t1], row_begin), ie = std::min(off[t1 + 1], row_end);
            // rows per scheduling chunk: small enough that a sampled row range
            // keeps every thread busy (rows are independent: any schedule
            // gives the same bits)
            int nth = 1;
#ifdef _OPENMP
            nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
            const int64_t csize = std::max<int64_t>(1, std::min<int64_t>(64, (ie - ib) / (8 * (int64_t)nth)));
#pragma omp parallel for schedule(dynamic, csize)
            for (int64_t gi = ib; gi < ie; ++gi) {
                const int64_t i = gi - off[t1];
                const double pix = pos[3 * gi], piy = pos[3 * gi + 1], piz = pos[3 * gi + 2];
                double fx = force[3 * gi], fy = force[3 * gi + 1], fz = force[3 * gi + 2];
                double pe = potential[gi], tt = temp[gi];
                for (int64_t j = 0; j < counts[t2]; ++j) {
                    if (t1 == t2 && i == j) continue;           // :178-180
                    const int64_t gj = off[t2] + j;
                    double rx = pos[3 * gj] - pix;                 // :181-185
                    double ry = pos[3 * gj + 1] - piy;
                    double rz = pos[3 * gj + 2] - piz;
                    if (rx < -bx / 2.0) rx += bx; else if (rx > bx / 2.0) rx -= bx;   // :186-200
                    if (ry < -by / 2.0) ry += by; else if (ry > by / 2.0) ry -= by;
                    if (rz < -bz / 2.0) rz += bz; else if (rz > bz / 2.0) rz -= bz;
                    const double r_abs = std::sqrt(rx * rx + ry * ry + rz * rz);   // :201
                    if (r_abs > r_cut) continue;                   // :202-204
                    double u, dudr;
                    lj_eval(pot, r_abs, &u, &dudr);                // :206
                    const double ffx = rx / r_abs * dudr;          // :207
                    const double ffy = ry / r_abs * dudr;
                    const double ffz = rz / r_abs * dudr;
                    const double t = ffx * rx + ffy * ry + ffz * rz;   // :208
                    fx += ffx; fy += ffy; fz += ffz;               // :209
                    pe += u;                                       // :210
                    tt += t;                                       // :211
                }
                force[3 * gi] = fx; force[3 * gi + 1] = fy; force[3 * gi + 2] = fz;
                potential[gi] = pe; temp[gi] = tt;
            }
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// macro_parameters (solver/src/macro_parameters/*.rs).  All sums are serial in
// atom order, as the reference's iterator folds are.

// mod.rs:12-25 get_center_of_mass_velocity
void oref_com_velocity(int ntypes, const int64_t* counts, const double* vel,
                       const double* mass_per_type, int type, double out[3]) {
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    const double m = mass_per_type[type];
    double sx = 0.0, sy = 0.0, sz = 0.0, sw = 0.0;
    for (int64_t k = 0; k < counts[type]; ++k) {
        const double* v = vel + 3 * (b + k);
        sx += v[0] * m; sy += v[1] * m; sz += v[2] * m; sw += 1.0 * m;
    }
    out[0] = sx / sw; out[1] = sy / sw; out[2] = sz / sw;
    (void)ntypes;
}

// mod.rs:28-34 get_momentum_of_system
void oref_momentum(int ntypes, const int64_t* counts, const double* vel,
                   const double* mass_per_type, int type, double out[3]) {
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    const double m = mass_per_type[type];
    double px = 0.0, py = 0.0, pz = 0.0;
    for (int64_t k = 0; k < counts[type]; ++k) {
        const double* v = vel + 3 * (b + k);
        px += v[0] * m; py += v[1] * m; pz += v[2] * m;
    }
    out[0] = px; out[1] = py; out[2] = pz;
    (void)ntypes;
}

// energy.rs:14-22 get_kinetic_energy: sum of m * (v.v) / 2
double oref_kinetic_energy(int ntypes, const int64_t* counts, const double* vel,
                           const double* mass_per_type, int type) {
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    const double m = mass_per_type[type];
    double s = 0.0;
    for (int64_t k = 0; k < counts[type]; ++k) {
        const double* v = vel + 3 * (b + k);
        s += m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / 2.0;
    }
    (void)ntypes;
    return s;
}

// energy.rs:25-37 get_thermal_energy: sum of m * |v - vcm|^2 / 2
double oref_thermal_energy(int ntypes, const int64_t* counts, const double* vel,
                           const double* mass_per_type, int type, const double vcm[3]) {
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    const double m = mass_per_type[type];
    double s = 0.0;
    for (int64_t k = 0; k < counts[type]; ++k) {
        const double* v = vel + 3 * (b + k);
        const double dx = v[0] - vcm[0], dy = v[1] - vcm[1], dz = v[2] - vcm[2];
        s += m * (dx * dx + dy * dy + dz * dz) / 2.0;
    }
    (void)ntypes;
    return s;
}

// energy.rs:40-49 get_potential_energy: sum(potential) / 2
double oref_potential_energy(int ntypes, const int64_t* counts, const double* potential, int type) {
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    double s = 0.0;
    for (int64_t k = 0; k < counts[type]; ++k) s += potential[b + k];
    (void)ntypes;
    return s / 2.0;
}

// pressure.rs:5-20 get_pressure
double oref_pressure(int ntypes, const int64_t* counts, const double* vel, const double* temp,
                     const double* mass_per_type, int type, const double vcm[3], const double box[3]) {
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    const double m = mass_per_type[type];
    const double volume = box[0] * box[1] * box[2];
    double r1 = 0.0, r2 = 0.0;
    for (int64_t k = 0; k < counts[type]; ++k) {
        const double* v = vel + 3 * (b + k);
        const double dx = v[0] - vcm[0], dy = v[1] - vcm[1], dz = v[2] - vcm[2];
        r1 += m * dx * dx;
        r1 += m * dy * dy;
        r1 += m * dz * dz;
        r2 -= temp[b + k];
    }
    (void)ntypes;
    return (r1 + r2 * 0.5) / volume / 3.0;
}

// temperature.rs:4-7 get_temperature
double oref_temperature(double thermal_energy, int64_t number_particles) {
    const double t = (2.0 * thermal_energy) / (3.0 * (double)number_particles * OREF_K_B);
    return t * 100.0;
}

// ---------------------------------------------------------------------------
// Coupling objects (mutable state, like the reference's enum fields).
enum { OREF_THERMO_BERENDSEN = 0, OREF_THERMO_NOSE_HOOVER = 1 };
struct oref_thermostat { int kind; double tau; double lambda; double psi; };
struct oref_barostat { double beta; double tau; double myu; };

static void temperature_of(int ntypes, const int64_t* counts, const double* vel,
                           const double* mass, int type, double* T) {
    double vcm[3];
    oref_com_velocity(ntypes, counts, vel, mass, type, vcm);
    const double e = oref_thermal_energy(ntypes, counts, vel, mass, type, vcm);
    *T = oref_temperature(e, counts[type]);
}

// thermostat.rs:24-45 calculate_lambda
static void thermo_calculate_lambda(oref_thermostat* th, int ntypes, const int64_t* counts,
                                    const double* vel, const double* mass, int type,
                                    double dt, double T0) {
    double T;
    temperature_of(ntypes, counts, vel, mass, type, &T);
    if (th->kind == OREF_THERMO_BERENDSEN) {
        const double l2 = 1.0 + dt / th->tau * (T0 / T - 1.0);
        th->lambda = std::sqrt(l2);
    } else {
        const double psi_dot = -((T0 / T) - 1.0) / th->tau;
        th->psi += psi_dot * (dt / 2.0);
        th->lambda = std::exp(-th->psi * dt / 2.0);
    }
}

// thermostat.rs:47-71 update
static void thermo_update(oref_thermostat* th, int ntypes, const int64_t* counts, double* vel,
                          const double* mass, int type, double dt, double T0) {
    double T;
    temperature_of(ntypes, counts, vel, mass, type, &T);
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    for (int64_t k = 0; k < counts[type]; ++k) {
        double* v = vel + 3 * (b + k);
        v[0] *= th->lambda; v[1] *= th->lambda; v[2] *= th->lambda;
    }
    if (th->kind == OREF_THERMO_NOSE_HOOVER) {
        const double psi_dot = -((T0 / T) - 1.0) / th->tau;
        th->psi += psi_dot * (dt / 2.0);
    }
}

// barostat.rs:21-36 calculate_myu
static void baro_calculate_myu(oref_barostat* ba, int ntypes, const int64_t* counts,
                               const double* vel, const double* temp, const double* mass,
                               const double box[3], int type, double dt, double P0) {
    double vcm[3];
    oref_com_velocity(ntypes, counts, vel, mass, type, vcm);
    const double P = oref_pressure(ntypes, counts, vel, temp, mass, type, vcm, box);
    const double m3 = 1.0 + dt * ba->beta / ba->tau * (P - P0);
    ba->myu = std::cbrt(m3);
}

// barostat.rs:39-49 update
static void baro_update(oref_barostat* ba, const int64_t* counts, double* pos, double box[3], int type) {
    box[0] *= ba->myu; box[1] *= ba->myu; box[2] *= ba->myu;
    int64_t b = 0;
    for (int t = 0; t < type; ++t) b += counts[t];
    for (int64_t k = 0; k < counts[type]; ++k) {
        double* p = pos + 3 * (b + k);
        p[0] *= ba->myu; p[1] *= ba->myu; p[2] *= ba->myu;
    }
}

// core/src/particle.rs:120-141 apply_boundary_conditions
void oref_apply_boundary_conditions(int64_t n, double* pos, const double box[3]) {
    for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            double& x = pos[3 * i + a];
            if (x < 0.0) x += box[a]; else if (x >= box[a]) x -= box[a];
        }
    }
}

// solver/src/solver/integrator.rs:14-59 VerletMethod::calculate, `nsteps` times.
// thermo / baro may be null (the reference's `None`).
int oref_step(int ntypes, const int64_t* counts, double* pos, double* vel, double* force,
              double* potential, double* temp, const double* mass_per_type, double box[3],
              const double* pot_table, double dt, int64_t nsteps,
              oref_barostat* baro, double P0, oref_thermostat* thermo, double T0, int nthreads) {
    int64_t n = 0;
    for (int t = 0; t < ntypes; ++t) n += counts[t];
    for (int64_t s = 0; s < nsteps; ++s) {
        if (baro)                                                   // :20-24
            for (int t = 0; t < ntypes; ++t)
                baro_calculate_myu(baro, ntypes, counts, vel, temp, mass_per_type, box, t, dt, P0);
        if (thermo)                                                 // :25-29
            for (int t = 0; t < ntypes; ++t)
                thermo_calculate_lambda(thermo, ntypes, counts, vel, mass_per_type, t, dt, T0);
        {                                                           // :30-36 kick
            int64_t b = 0;
            for (int t = 0; t < ntypes; ++t) {
                const double c = dt / (2.0 * mass_per_type[t]);
                for (int64_t k = 0; k < counts[t]; ++k) {
                    double* v = vel + 3 * (b + k); const double* f = force + 3 * (b + k);
                    v[0] = v[0] + f[0] * c; v[1] = v[1] + f[1] * c; v[2] = v[2] + f[2] * c;
                }
                b += counts[t];
            }
        }
        if (thermo)                                                 // :37-41
            for (int t = 0; t < ntypes; ++t)
                thermo_update(thermo, ntypes, counts, vel, mass_per_type, t, dt, T0);
        for (int64_t i = 0; i < n; ++i)                             // :42-46 drift
            for (int a = 0; a < 3; ++a) pos[3 * i + a] += vel[3 * i + a] * dt;
        oref_apply_boundary_conditions(n, pos, box);                // :47
        oref_update_force(ntypes, counts, pos, box, pot_table, force, potential, temp,
                          nthreads, 0, -1);                         // :48
        {                                                           // :49-55 kick
            int64_t b = 0;
            for (int t = 0; t < ntypes; ++t) {
                const double c = dt / (2.0 * mass_per_type[t]);
                for (int64_t k = 0; k < counts[t]; ++k) {
                    double* v = vel + 3 * (b + k); const double* f = force + 3 * (b + k);
                    v[0] += f[0] * c; v[1] += f[1] * c; v[2] += f[2] * c;
                }
                b += counts[t];
            }
        }
        if (baro)                                                   // :56-60
            for (int t = 0; t < ntypes; ++t) baro_update(baro, counts, pos, box, t);
    }
    return 0;
}

// solver/src/initializer/position.rs:34-99: U and FCC fill order.
// kind 0 = U (1 site per cell), 1 = FCC (4 sites per cell).
int oref_lattice(int kind, int64_t nx, int64_t ny, int64_t nz, double a,
                 const double start[3], double* pos) {
    for (int64_t x = 0; x < nx; ++x)
        for (int64_t y = 0; y < ny; ++y)
            for (int64_t z = 0; z < nz; ++z) {
                const int64_t cell = x * ny * nz + y * nz + z;
                if (kind == 0) {
                    double* p = pos + 3 * cell;
                    p[0] = start[0] + (double)x * a; p[1] = start[1] + (double)y * a;
                    p[2] = start[2] + (double)z * a;
                } else {
                    double* p = pos + 3 * (cell * 4);
                    p[0] = start[0] + (double)x * a; p[1] = start[1] + (double)y * a;
                    p[2] = start[2] + (double)z * a;
                    p[3] = start[0] + (double)x * a; p[4] = start[1] + ((double)y + 0.5) * a;
                    p[5] = start[2] + ((double)z + 0.5) * a;
                    p[6] = start[0] + ((double)x + 0.5) * a; p[7] = start[1] + (double)y * a;
                    p[8] = start[2] + ((double)z + 0.5) * a;
                    p[9] = start[0] + ((double)x + 0.5) * a; p[10] = start[1] + ((double)y + 0.5) * a;
                    p[11] = start[2] + (double)z * a;
                }
            }
    return 0;
}

// The set of pairs update_force sums (potential.rs:171-204): (i, j) flat
// indices, i of type t1, j of type t2 >= t1, j != i, with the reference's
// single-shift minimum image and |r| <= r_cut.  Writes up to `capacity`
// pairs, returns the total count.
int64_t oref_pairs(int ntypes, const int64_t* counts, const double* pos, const double box[3],
                   const double* pot_table, int64_t capacity, int32_t* out_i, int32_t* out_j) {
    std::vector<int64_t> off(ntypes + 1, 0);
    for (int t = 0; t < ntypes; ++t) off[t + 1] = off[t] + counts[t];
    const double bx = box[0], by = box[1], bz = box[2];
    int64_t total = 0;
    for (int t1 = 0; t1 < ntypes; ++t1)
        for (int t2 = t1; t2 < ntypes; ++t2) {
            const double r_cut = table_get(pot_table, ntypes, t1, t2).r_cut;
            for (int64_t gi = off[t1]; gi < off[t1 + 1]; ++gi)
                for (int64_t gj = off[t2]; gj < off[t2 + 1]; ++gj) {
                    if (gi == gj) continue;
                    double rx = pos[3 * gj] - pos[3 * gi];
                    double ry = pos[3 * gj + 1] - pos[3 * gi + 1];
                    double rz = pos[3 * gj + 2] - pos[3 * gi + 2];
                    if (rx < -bx / 2.0) rx += bx; else if (rx > bx / 2.0) rx -= bx;
                    if (ry < -by / 2.0) ry += by; else if (ry > by / 2.0) ry -= by;
                    if (rz < -bz / 2.0) rz += bz; else if (rz > bz / 2.0) rz -= bz;
                    if (std::sqrt(rx * rx + ry * ry + rz * rz) > r_cut) continue;
                    if (total < capacity) { out_i[total] = (int32_t)gi; out_j[total] = (int32_t)gj; }
                    ++total;
                }
        }
    return total;
}

int oref_abi_version(void) { return 1; }

}  // extern "C"
