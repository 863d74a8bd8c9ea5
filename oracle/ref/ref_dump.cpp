// Oracle pinning harness (test infrastructure only; never part of the product).
//
// Drives the reference oxDNA CPU code through its own public classes (SimManager,
// ConfigInfo, BaseInteraction) and prints, in %.17g:
//   * the state the reference holds after initialisation (positions after its strand
//     centre-of-mass shift, the orthonormalised frame a1 a2 a3, bonds, types);
//   * per-particle forces (lab frame) and torques (body frame) from one full force
//     evaluation, accumulated exactly as MD_CPUBackend::_compute_forces does
//     (src/Backends/MD_CPUBackend.cpp:146-167): the external forces of the current step, bonded
//     pairs through `affected`, then every non-bonded pair once with the higher index first
//     (src/Lists/Cells.cpp:168);
//   * the per-term energy split (src/Interactions/BaseInteraction.cpp:61-86);
//   * when the input asks for steps > 0, the state after SimManager::run().
//
// usage: ref_dump <input file> <output file> [key=value ...]

#include "Managers/SimManager.h"
#include "Utilities/ConfigInfo.h"
#include "Utilities/Logger.h"
#include "Utilities/Timings.h"
#include "Interactions/BaseInteraction.h"
#include "Particles/BaseParticle.h"
#include "Boxes/BaseBox.h"

#include <cstdio>
#include <string>
#include <vector>

static void dump_state(FILE *out, const char *tag, bool with_momenta) {
	auto &ps = CONFIG_INFO->particles();
	fprintf(out, "%s %zu\n", tag, ps.size());
	for(auto p : ps) {
		const LR_vector &a1 = p->orientationT.v1, &a2 = p->orientationT.v2, &a3 = p->orientationT.v3;
		fprintf(out, "%.17g %.17g %.17g  %.17g %.17g %.17g  %.17g %.17g %.17g  %.17g %.17g %.17g",
				p->pos.x, p->pos.y, p->pos.z, a1.x, a1.y, a1.z, a2.x, a2.y, a2.z, a3.x, a3.y, a3.z);
		if(with_momenta) {
			fprintf(out, "  %.17g %.17g %.17g  %.17g %.17g %.17g", p->vel.x, p->vel.y, p->vel.z, p->L.x, p->L.y, p->L.z);
		}
		fprintf(out, "\n");
	}
}

int main(int argc, char *argv[]) {
	if(argc < 3) {
		fprintf(stderr, "usage: %s input_file output_file [key=value ...]\n", argv[0]);
		return 2;
	}
	try {
		Logger::init();
		TimingManager::init();

		input_file input(true);
		input.init_from_filename(argv[1]);
		for(int i = 3; i < argc; i++) {
			input.init_from_string(argv[i]);
		}

		SimManager sim(input);
		sim.load_options();
		sim.init();

		FILE *out = fopen(argv[2], "w");
		if(out == nullptr) {
			fprintf(stderr, "cannot open %s\n", argv[2]);
			return 2;
		}

		auto &ps = CONFIG_INFO->particles();
		BaseInteraction *inter = CONFIG_INFO->interaction;
		LR_vector sides = CONFIG_INFO->box->box_sides();
		fprintf(out, "box %.17g %.17g %.17g\n", sides.x, sides.y, sides.z);
		fprintf(out, "rcut %.17g\n", inter->get_rcut());
		fprintf(out, "topology %zu\n", ps.size());
		for(auto p : ps) {
			fprintf(out, "%d %d %d %d %d\n", p->n3 ? p->n3->index : -1, p->n5 ? p->n5->index : -1, p->type, p->btype, p->strand_id);
		}
		dump_state(out, "state", true);

		// forces start from the external forces, as in MD_CPUBackend::_compute_forces
		// (src/Backends/MD_CPUBackend.cpp:146-155); zero without external forces
		for(auto p : ps) {
			p->force = LR_vector(0., 0., 0.);
			p->torque = LR_vector(0., 0., 0.);
			p->set_initial_forces(CONFIG_INFO->curr_step, CONFIG_INFO->box);
		}
		fprintf(out, "step %lld\n", (long long) CONFIG_INFO->curr_step);
		inter->begin_energy_and_force_computation();
		number U = 0.;
		for(auto p : ps) {
			for(auto &pair : p->affected) {
				if(pair.first == p) {
					U += inter->pair_interaction_bonded(pair.first, pair.second, true, true);
				}
			}
		}
		for(size_t i = 0; i < ps.size(); i++) {
			for(size_t j = 0; j < i; j++) {
				U += inter->pair_interaction_nonbonded(ps[i], ps[j], true, true);
			}
		}
		fprintf(out, "forces %zu\n", ps.size());
		for(auto p : ps) {
			fprintf(out, "%.17g %.17g %.17g  %.17g %.17g %.17g\n", p->force.x, p->force.y, p->force.z, p->torque.x, p->torque.y, p->torque.z);
		}
		fprintf(out, "energy %.17g\n", U);

		auto split = inter->get_system_energy_split(ps, CONFIG_INFO->lists);
		fprintf(out, "split %zu\n", split.size());
		for(auto &kv : split) {
			fprintf(out, "%d %.17g\n", kv.first, kv.second);
		}

		int steps = 0;
		getInputInt(&input, "steps", &steps, 0);
		if(steps > 0) {
			sim.run();
			dump_state(out, "final", true);
		}
		fclose(out);
	}
	catch(oxDNAException &e) {
		fprintf(stderr, "reference error: %s\n", e.what());
		return 1;
	}
	return 0;
}
