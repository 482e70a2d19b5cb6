// Reads a MolFlow+ file through the C++ adapter (mfg::XmlFile) and prints what the host sees:
// facet and moment counts, the stored global counters and the sums of the stored facet counters.
// With a third argument, writes the model and the stored results back to that path (mfg_xml_save).
// Usage: xml_check <file.xml|file.zip> [catalog folder or ""] [output file]
#include <cstdio>

#include "mfg_simulation.hpp"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    try {
        mfg::XmlFile file(argv[1], argc > 2 && argv[2][0] ? argv[2] : nullptr);
        const mfg_model_desc& d = file.desc();
        mfg_model* model = nullptr;
        mfg::check(mfg_model_create(&d, &model));
        std::printf("facets %d moments %d params %d results %d\n", d.n_facets, d.n_moments, d.n_params,
                    int(file.has_results()));
        if (file.has_results()) {
            mfg::HostState st;
            mfg::ReadStoredResults(file, model, st);
            unsigned long long hits = 0, des = 0;
            for (size_t i = 0; i < st.facet_counts.size(); i += MFG_FC_N) {
                hits += st.facet_counts[i + MFG_FC_NBMCHIT];
                des += st.facet_counts[i + MFG_FC_NBDESORBED];
            }
            std::printf("global %.17g %.17g %.17g facet_hits %llu facet_des %llu\n", st.global[MFG_G_NBMCHIT],
                        st.global[MFG_G_NBDESORBED], st.global[MFG_G_NBLEAK], hits, des);
            if (argc > 3) {
                mfg_state_view v = st.view();
                mfg::check(mfg_xml_save(argv[3], &d, model, &v, nullptr));
                std::printf("saved %s\n", argv[3]);
            }
        }
        mfg_model_destroy(model);
    } catch (const mfg::Error& e) {
        std::printf("error %d %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
