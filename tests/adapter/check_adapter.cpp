// Compiles the GB300 adapter (nbody_gb300/adapter/nbody_engine_gb300.h)
// against the reference's own nbody_engine.h and links it with the
// reference's objects and libnbody_gb300.so: the drop-in the solvers would
// use is type-checked against nbody/nbody_engine.h:16-96 and every symbol
// resolves.  Run without a GPU it checks the factory's answers: NULL for an
// invalid parameter and NULL when no engine can be created.  With a GPU it
// also steps a reference solver on the adapter (rk4, 64 bodies) and compares
// with the reference's simple engine.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "nbody_engine_gb300.h"
#include "nbody_engines.h"
#include "nbody_solvers.h"

static QVariantMap params(std::initializer_list<std::pair<const char*, const char*>> kv)
{
	QVariantMap m;
	for(const auto& p : kv) { m[QString(p.first)] = QVariant(QString(p.second)); }
	return m;
}

int main(int argc, char** argv)
{
	const bool have_gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
	// invalid values: NULL, like the reference's factory
	if(nbody_create_engine_gb300(params({{"device", "x"}})) != nullptr) { return 1; }
	if(nbody_create_engine_gb300(params({{"algo", "tree"}})) != nullptr) { return 2; }
	if(nbody_create_engine_gb300(params({{"tree_layout", "tree"}})) != nullptr) { return 3; }
	nbody_engine* e = nbody_create_engine_gb300(params({{"precision", "fp64"}}));
	if(!have_gpu)
	{
		if(e != nullptr) { return 4; }  // no device: no engine
		std::printf("adapter ok (no GPU)\n");
		return 0;
	}
	if(e == nullptr) { return 5; }
	nbody_data d1, d2;
	d1.make_universe(32, 100, 100, 100);
	d2.make_universe(32, 100, 100, 100);
	nbody_engine* ref = nbody_create_engine(params({{"engine", "simple"}}));
	nbody_solver* s1 = nbody_create_solver(params({{"solver", "rk4"}}));
	nbody_solver* s2 = nbody_create_solver(params({{"solver", "rk4"}}));
	if(!e->init(&d1) || !ref->init(&d2)) { return 6; }
	s1->set_engine(e);
	s2->set_engine(ref);
	s1->run(&d1, nullptr, 0.05, 0, 0);
	s2->run(&d2, nullptr, 0.05, 0, 0);
	e->get_data(&d1);
	ref->get_data(&d2);
	const bool same = d1.is_equal(d2, 1e-12);
	delete s1;
	delete s2;
	delete e;
	delete ref;
	std::printf("adapter rk4 vs simple: %s\n", same ? "equal" : "DIFFERENT");
	return same ? 0 : 7;
}
