// nbody_engine_gb300.h -- the reference-side drop-in for the GB300 engine.
//
// A maintainer of drons/nbody adds this header to nbody/ and one branch to
// nbody_create_engine (nbody/nbody_engines.cpp:4-193):
//
//     #ifdef HAVE_GB300
//     else if(type == "gb300") { return nbody_create_engine_gb300(param); }
//     #endif
//
// nbody_engine_gb300 subclasses the reference's abstract engine
// (nbody/nbody_engine.h:16-96) and forwards every virtual to the C ABI of
// libnbody_gb300.so (include/nbody_gb300.h), so every solver drives it
// unchanged.  nbody_data_stream_gb300 is the frame stream writer
// (nbody/nbody_data_stream.h) that writes straight from the engine's device
// state.  Everything is inline; it needs the reference's headers, Qt's
// QDebug / QString / QVariantMap and libnbody_gb300.so.
#ifndef NBODY_ENGINE_GB300_H
#define NBODY_ENGINE_GB300_H

#include <QDebug>
#include <QString>
#include <QVariantMap>
#include <vector>

#include "nbody_data_stream.h"
#include "nbody_engine.h"
#include "nbody_gb300.h"

class nbody_engine_gb300 : public nbody_engine
{
	nbg_engine*		m_e = nullptr;
	nbody_data*		m_data = nullptr;

	// one engine buffer
	class smemory : public memory
	{
	public:
		nbg_buffer*	b;
		explicit smemory(nbg_buffer* x) : b(x) {}
		size_t size() const override { return nbg_buffer_size(b); }
	};
	smemory*		m_y = nullptr;

	// foreign memory -> NULL handle, which every entry point rejects with a
	// status and no side effect (the reference's "is not smemory" branch)
	static nbg_buffer* buf(const memory* m)
	{
		const smemory* s = dynamic_cast<const smemory*>(m);
		return s != nullptr ? s->b : nullptr;
	}
	static std::vector<const nbg_buffer*> bufs(const memory_array& a)
	{
		std::vector<const nbg_buffer*> out;
		for(const memory* m : a) { out.push_back(buf(m)); }
		return out;
	}
	void check(nbg_status st, const char* what) const
	{
		if(st != NBG_OK) { qDebug() << what << nbg_status_string(st) << nbg_last_error(m_e); }
	}

public:
	explicit nbody_engine_gb300(const nbg_params& p) { nbg_engine_create(&p, &m_e); }
	~nbody_engine_gb300() override
	{
		delete m_y;
		nbg_engine_destroy(m_e);
	}
	bool valid() const { return m_e != nullptr; }
	nbg_engine* handle() const { return m_e; }

	const char* type_name() const override { return nbg_type_name(m_e); }
	bool init(nbody_data* d) override
	{
		m_data = d;
		if(nbg_init(m_e, d->get_count(), &d->get_vertites()->x, &d->get_velosites()->x,
					d->get_mass()) != NBG_OK)
		{
			qDebug() << "gb300 init:" << nbg_last_error(m_e);
			return false;
		}
		delete m_y;
		m_y = new smemory(nbg_get_y(m_e));
		return true;
	}
	void get_data(nbody_data* d) override
	{
		check(nbg_get_data(m_e, &d->get_vertites()->x, &d->get_velosites()->x), "get_data");
	}
	size_t problem_size() const override { return nbg_problem_size(m_e); }
	memory* get_y() override { return m_y; }
	void advise_time(const nbcoord_t& dt) override { m_data->advise_time(dt); }
	nbcoord_t get_time() const override { return m_data->get_time(); }
	void set_time(nbcoord_t t) override { m_data->set_time(t); }
	size_t get_step() const override { return m_data->get_step(); }
	void set_step(size_t s) override { m_data->set_step(s); }

	void fcompute(const nbcoord_t& t, const memory* y, memory* f) override
	{
		advise_compute_count();
		check(nbg_fcompute(m_e, t, m_data->get_step(), buf(y), buf(f)), "fcompute");
	}
	void clamp(memory* y, nbcoord_t b) override { check(nbg_clamp(m_e, buf(y), b), "clamp"); }

	memory* create_buffer(size_t s) override
	{
		nbg_buffer* b = nullptr;
		return nbg_create_buffer(m_e, s, &b) == NBG_OK ? new smemory(b) : nullptr;
	}
	void free_buffer(memory* m) override
	{
		if(smemory* s = dynamic_cast<smemory*>(m)) { nbg_free_buffer(m_e, s->b); }
		delete m;
	}
	void read_buffer(void* dst, const memory* src) override
	{
		check(nbg_read_buffer(m_e, dst, buf(src)), "read_buffer");
	}
	void write_buffer(memory* dst, const void* src) override
	{
		check(nbg_write_buffer(m_e, buf(dst), src), "write_buffer");
	}
	void copy_buffer(memory* a, const memory* b) override
	{
		check(nbg_copy_buffer(m_e, buf(a), buf(b)), "copy_buffer");
	}
	void fill_buffer(memory* a, const nbcoord_t& v) override
	{
		check(nbg_fill_buffer(m_e, buf(a), v), "fill_buffer");
	}
	void fmadd_inplace(memory* a, const memory* b, const nbcoord_t& c) override
	{
		check(nbg_fmadd_inplace(m_e, buf(a), buf(b), c), "fmadd_inplace");
	}
	void fmadd(memory* a, const memory* b, const memory* c, const nbcoord_t& d) override
	{
		check(nbg_fmadd(m_e, buf(a), buf(b), buf(c), d), "fmadd");
	}
	void fmaddn_inplace(memory* a, const memory_array& b, const nbcoord_t* c,
						size_t csize) override
	{
		const std::vector<const nbg_buffer*> bb(bufs(b));
		check(nbg_fmaddn_inplace(m_e, buf(a), bb.data(), bb.size(), c, csize), "fmaddn_inplace");
	}
	void fmaddn_corr(memory* a, memory* corr, const memory_array& b, const nbcoord_t* c,
					 size_t csize) override
	{
		const std::vector<const nbg_buffer*> bb(bufs(b));
		check(nbg_fmaddn_corr(m_e, buf(a), buf(corr), bb.data(), bb.size(), c, csize),
			  "fmaddn_corr");
	}
	void fmaddn(memory* a, const memory* b, const memory_array& c, const nbcoord_t* d,
				size_t dsize) override
	{
		const std::vector<const nbg_buffer*> cc(bufs(c));
		check(nbg_fmaddn(m_e, buf(a), b != nullptr ? buf(b) : nullptr, cc.data(), cc.size(), d,
						 dsize), "fmaddn");
	}
	void fmaxabs(const memory* a, nbcoord_t& result) override
	{
		check(nbg_fmaxabs(m_e, buf(a), &result), "fmaxabs");
	}
	void print_info() const override
	{
		qDebug() << "\tengine:" << nbg_type_name(m_e);
	}
};

// The factory branch: the engine keys of nbody_create_engine plus the GB300
// ones, NULL on an invalid value or when the engine cannot be created (no
// GPU, device out of range), as the reference's factory answers.
inline nbody_engine* nbody_create_engine_gb300(const QVariantMap& param)
{
	nbg_params p;
	nbg_params_default(&p);
	bool ok = false;
	p.device = param.value("device", "0").toString().toInt(&ok);
	if(!ok) { return nullptr; }
	const QString algo(param.value("algo", "direct").toString());
	const QString prec(param.value("precision", "fp64").toString());
	const QString layout(param.value("tree_layout", "heap_stackless").toString());
	const QString trav(param.value("traverse_type", "nested_tree").toString());
	if(!(algo == "direct" || algo == "bh") || !(prec == "fp64" || prec == "mixed") ||
	   !(layout == "heap" || layout == "heap_stackless") ||
	   !(trav == "cycle" || trav == "nested_tree"))
	{
		return nullptr;
	}
	p.algo = algo == "bh" ? NBG_ALGO_BH : NBG_ALGO_DIRECT;
	p.precision = prec == "mixed" ? NBG_PREC_MIXED : NBG_PREC_FP64;
	p.tree_layout = layout == "heap" ? NBG_LAYOUT_HEAP : NBG_LAYOUT_HEAP_STACKLESS;
	p.traverse_type = trav == "cycle" ? NBG_TRAVERSE_CYCLE : NBG_TRAVERSE_NESTED_TREE;
	p.softening = param.value("softening", 0.0).toDouble();
	p.distance_to_node_radius_ratio = param.value("distance_to_node_radius_ratio", 10).toDouble();
	p.tree_build_rate = param.value("tree_build_rate", 0).toULongLong();
	p.learned = param.value("learned", false).toBool() ? 1 : 0;
	p.learned_tight_ratio = param.value("learned_tight_ratio", 2.0).toDouble();
	nbody_engine_gb300* e = new nbody_engine_gb300(p);
	if(!e->valid())
	{
		delete e;
		return nullptr;
	}
	if(param.contains("tree_refit_within_step"))
	{
		nbg_tune_set(e->handle(), "bh.refit_within_step",
					 param.value("tree_refit_within_step").toBool() ? 1 : 0);
	}
	if(param.contains("tree_freeze_within_step"))
	{
		nbg_tune_set(e->handle(), "bh.freeze_within_step",
					 param.value("tree_freeze_within_step").toBool() ? 1 : 0);
	}
	if(param.contains("learned_judge"))
	{
		nbg_tune_set(e->handle(), "learned.judge", param.value("learned_judge").toBool() ? 1 : 0);
	}
	if(param.contains("learned_judge_samples"))
	{
		const int samples = param.value("learned_judge_samples").toInt();
		if(samples < 1)	// the Python factory's answer to the same value
		{
			delete e;
			return nullptr;
		}
		nbg_tune_set(e->handle(), "learned.judge_samples", samples);
	}
	return e;
}

// Frame stream writer from the engine's device state (same file format as
// nbody_data_stream, nbody/nbody_data_stream.cpp:62-229): the solver's run
// loop can skip get_data before write.
class nbody_data_stream_gb300 : public nbody_data_stream
{
	nbg_engine*			m_e;
	nbg_stream_writer*	m_w = nullptr;
	bool				m_header = false;
public:
	explicit nbody_data_stream_gb300(nbg_engine* e) : m_e(e) {}
	~nbody_data_stream_gb300() override
	{
		if(m_w != nullptr) { nbg_stream_close(m_w); }
	}
	int open_gb300(const QString& name, qint64 max_part_size, bool append)
	{
		if(m_w != nullptr) { nbg_stream_close(m_w); }
		m_w = nullptr;
		m_header = false;
		return nbg_stream_open(m_e, name.toStdString().c_str(), max_part_size, append ? 1 : 0,
							   &m_w) == NBG_OK ? 0 : -1;
	}
	int write(const nbody_data* d) override
	{
		if(d == nullptr || m_w == nullptr) { return -1; }
		if(!m_header)
		{
			m_header = nbg_stream_set_header(m_w, d->get_count(), d->get_box_size(),
											 reinterpret_cast<const float*>(d->get_color()),
											 d->get_mass()) == NBG_OK;
		}
		return nbg_stream_write(m_w, nbg_get_y(m_e), d->get_step(), d->get_time()) == NBG_OK
			   ? 0 : -1;
	}
};

#endif // NBODY_ENGINE_GB300_H
