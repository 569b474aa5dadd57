// ref_glue.cpp -- a C ABI over the reference's own CPU code, compiled from the
// reference's sources (nbody/*.cpp, unchanged) against the Qt-API shim in
// oracle/qtshim into oracle/_ref/libnbody_ref.so by oracle/ref_build.py.
//
// TEST INFRASTRUCTURE ONLY: it lets the tests check the oracle restatement
// (oracle/nbody_oracle.c) and the GB300 engine's fixtures against what the
// reference itself computes.  Nothing in the GB300 engine links or loads it,
// and it is built only where the reference's sources are present.
//
// Every entry point works like the reference's own tests drive the code:
//  * ref_make_universe     nbody_data::make_universe (nbody/nbody_data.cpp:263-324)
//  * ref_fcompute          nbody_create_engine (nbody/nbody_engines.cpp:4-193) +
//                          the fcompute loop of test_nbody_engine_compare
//                          (test/engine/test_nbody_engine.cpp:472-550):
//                          poisoned f, set_step, fcompute, y *= (1 + mutate)
//  * ref_solver_run        nbody_create_solver (nbody/nbody_solvers.cpp:17-110) +
//                          nbody_solver::run (test/solver/test_nbody_solver.cpp:43-85)
//  * ref_butcher_table     the table of a Butcher solver (nbody_solver_rk_butcher::table)
//  * ref_heap_build        nbody_space_heap::build and its node arrays
//  * ref_stream_write      nbody_data_stream::open / write / close
//  * ref_statistics        nbody_data::print_statistics' P, L, E, V sums
// Inputs and outputs use the engines' SoA state layout
// y = [rx | ry | rz | vx | vy | vz] (nbody/nbody_engine_simple.cpp:34-39).
#include <cstdint>
#include <cstring>
#include <string>

#include "nbody_butcher_table.h"
#include "nbody_data.h"
#include "nbody_data_stream.h"
#include "nbody_engine.h"
#include "nbody_engines.h"
#include "nbody_solver.h"
#include "nbody_solver_rk_butcher.h"
#include "nbody_solvers.h"
#include "nbody_space_heap.h"

namespace {

// "key=value;key=value" -> the factories' parameter map
QVariantMap parse_params(const char* kv) {
    QVariantMap m;
    std::string s(kv ? kv : "");
    size_t start = 0;
    while (start <= s.size()) {
        const size_t end = s.find(';', start);
        const std::string item = s.substr(start, end == std::string::npos ? std::string::npos
                                                                          : end - start);
        const size_t eq = item.find('=');
        if (eq != std::string::npos)
            m[QString(item.substr(0, eq))] = QVariant(QString(item.substr(eq + 1)));
        if (end == std::string::npos) break;
        start = end + 1;
    }
    return m;
}

void fill_data(nbody_data& d, size_t n, const double* y, const double* mass) {
    const nbcolor_t white(1, 1, 1, 1);
    for (size_t i = 0; i < n; ++i)
        d.add_body(nbvertex_t(y[i], y[n + i], y[2 * n + i]),
                   nbvertex_t(y[3 * n + i], y[4 * n + i], y[5 * n + i]), mass[i], white, 0);
}

void read_data(const nbody_data& d, double* y) {
    const size_t n = d.get_count();
    const nbvertex_t* r = d.get_vertites();
    const nbvertex_t* v = d.get_velosites();
    for (size_t i = 0; i < n; ++i) {
        y[i] = r[i].x;
        y[n + i] = r[i].y;
        y[2 * n + i] = r[i].z;
        y[3 * n + i] = v[i].x;
        y[4 * n + i] = v[i].y;
        y[5 * n + i] = v[i].z;
    }
}

}  // namespace

extern "C" {

// Two galaxies of round_up(star_count, 64) bodies each; *count = bodies.
// With cap >= *count the state and masses are written to y (6 count) and mass.
int ref_make_universe(size_t star_count, double sx, double sy, double sz, size_t cap, double* y,
                      double* mass, size_t* count) {
    nbody_data d;
    d.make_universe(star_count, sx, sy, sz);
    const size_t n = d.get_count();
    if (count) *count = n;
    if (cap < n || y == nullptr || mass == nullptr) return 0;
    read_data(d, y);
    std::memcpy(mass, d.get_mass(), n * sizeof(double));
    return 0;
}

// `steps` fcomputes of the engine the factory makes from engine_kv; after
// each, y *= (1 + mutate) through fmadd_inplace(y, y, mutate) when mutate != 0
// (test_fcompute uses 0.99).  f_out: steps x 6n.  Returns 0, or -1 when the
// factory rejects the parameters, -2 when init fails.
int ref_fcompute(const char* engine_kv, size_t n, const double* y0, const double* mass,
                 size_t steps, double mutate, double* f_out) {
    nbody_data d;
    fill_data(d, n, y0, mass);
    nbody_engine* e = nbody_create_engine(parse_params(engine_kv));
    if (e == nullptr) return -1;
    if (!e->init(&d)) {
        delete e;
        return -2;
    }
    nbody_engine::memory* f = e->create_buffer(sizeof(double) * e->problem_size());
    for (size_t s = 0; s < steps; ++s) {
        e->fill_buffer(f, (s % 2) ? 1e10 : -1e10);  // outputs the engine never writes show up
        e->set_step(s);
        e->fcompute(0, e->get_y(), f);
        e->read_buffer(f_out + s * 6 * n, f);
        if (mutate != 0.0) e->fmadd_inplace(e->get_y(), e->get_y(), mutate);
    }
    e->free_buffer(f);
    delete e;
    return 0;
}

// Solver from solver_kv driving the engine from engine_kv from t = 0 to
// max_time (nbody_solver::run without stream or checks); y_out = final state.
int ref_solver_run(const char* solver_kv, const char* engine_kv, size_t n, const double* y0,
                   const double* mass, double max_time, double* y_out, double* t_out,
                   uint64_t* steps_out) {
    nbody_data d;
    fill_data(d, n, y0, mass);
    nbody_engine* e = nbody_create_engine(parse_params(engine_kv));
    if (e == nullptr) return -1;
    nbody_solver* s = nbody_create_solver(parse_params(solver_kv));
    if (s == nullptr) {
        delete e;
        return -3;
    }
    if (!e->init(&d)) {
        delete s;
        delete e;
        return -2;
    }
    s->set_engine(e);
    s->run(&d, nullptr, max_time, 0, 0.0);
    e->get_data(&d);
    read_data(d, y_out);
    if (t_out) *t_out = d.get_time();
    if (steps_out) *steps_out = d.get_step();
    delete s;
    delete e;
    return 0;
}

// The Butcher table of the solver the factory makes from solver_kv:
// *steps = s; with cap >= s: a [s][s] row-major (zero above the diagonal of
// an explicit table), b1 [s], b2 [s], c [s], flags = 1 implicit | 2
// embedded.  -3: not a Butcher solver.
int ref_butcher_table(const char* solver_kv, size_t cap, size_t* steps, double* a, double* b1,
                      double* b2, double* c, int* flags) {
    nbody_solver* s = nbody_create_solver(parse_params(solver_kv));
    const nbody_solver_rk_butcher* rk = dynamic_cast<const nbody_solver_rk_butcher*>(s);
    // the solver's destructor frees its buffers through its engine: give it one
    nbody_engine* e = nbody_create_engine(parse_params("engine=simple"));
    if (s != nullptr) s->set_engine(e);
    if (rk == nullptr) {
        delete s;
        delete e;
        return -3;
    }
    const nbody_butcher_table* bt = rk->table();
    const size_t k = bt->get_steps();
    *steps = k;
    if (cap >= k) {
        const nbcoord_t** A = bt->get_a();
        const bool implicit = bt->is_implicit();
        for (size_t i = 0; i < k; ++i) {
            // explicit tables keep row i as its i entries below the diagonal
            for (size_t j = 0; j < k; ++j) a[i * k + j] = (implicit || j < i) ? A[i][j] : 0.0;
            b1[i] = bt->get_b1()[i];
            b2[i] = bt->get_b2()[i];
            c[i] = bt->get_c()[i];
        }
        *flags = (bt->is_implicit() ? 1 : 0) | (bt->is_embedded() ? 2 : 0);
    }
    delete s;
    delete e;
    return 0;
}

// kd heap of n bodies at ratio lambda: 2n entries (index 0 unused) of mass
// centre (3 x 2n, SoA), mass, crit r^2 and body index.
int ref_heap_build(size_t n, const double* y, const double* mass, double lambda, double* com,
                   double* nmass, double* r2, int64_t* body_n) {
    nbody_space_heap h;
    h.build(n, y, y + n, y + 2 * n, mass, lambda);
    const auto& mc = h.get_mass_center();
    const auto& m = h.get_mass();
    const auto& r = h.get_radius_sqr();
    const auto& b = h.get_body_n();
    const size_t sz = b.size();
    if (sz != 2 * n) return -1;
    for (size_t i = 0; i < sz; ++i) {
        com[i] = mc[i].x;
        com[sz + i] = mc[i].y;
        com[2 * sz + i] = mc[i].z;
        nmass[i] = m[i];
        r2[i] = r[i];
        body_n[i] = (int64_t)b[i];
    }
    return 0;
}

// Frames k = 0 .. frames-1 of n bodies (y_frames: frames x 6n, SoA) written
// with step[k], time[k] through nbody_data_stream (white colours, masses).
int ref_stream_write(const char* base, long long max_part_size, size_t n, size_t frames,
                     const double* y_frames, const double* mass, const uint64_t* step,
                     const double* time) {
    nbody_data_stream st;
    if (st.open(QString(base), max_part_size) != 0) return -1;
    for (size_t k = 0; k < frames; ++k) {
        nbody_data d;
        fill_data(d, n, y_frames + k * 6 * n, mass);
        d.set_step(step[k]);
        d.set_time(time[k]);
        if (st.write(&d) != 0) return -2;
    }
    st.close();
    return 0;
}

// print_statistics' conservation sums of one state (nbody/nbody_data.cpp:57-145):
// out = P[3], L[3], mass centre[3], KE, PE, total energy
int ref_statistics(size_t n, const double* y, const double* mass, double* out) {
    nbody_data d;
    fill_data(d, n, y, mass);
    d.set_check_list("PLVE");
    nbody_engine* e = nbody_create_engine(parse_params("engine=simple"));
    if (e == nullptr || !e->init(&d)) {
        delete e;
        return -1;
    }
    d.print_statistics(e);  // the first call records the initial values
    const nbvertex_t p = d.get_initial_impulce(), l = d.get_initial_impulce_moment();
    const nbvertex_t c = d.get_initial_mass_center();
    const double v[10] = {p.x, p.y, p.z, l.x, l.y, l.z, c.x, c.y, c.z, d.get_initial_energy()};
    for (int k = 0; k < 10; ++k) out[k] = v[k];
    delete e;
    return 0;
}

}  // extern "C"
