/*
 * Reference harness (TEST INFRASTRUCTURE ONLY — never linked into the product).
 *
 * Links the UNMODIFIED SCORE reference sources (compiled from their own files by
 * oracle/ref/Makefile) and drives their recrystallization-growth functions on a
 * host-generated domain, so that the reference itself produces the golden outputs
 * the CUDA path is checked against.
 *
 * Input injection (the reference can only synthesise cuboid/EBSD structures):
 *   - the deformed-grain label grid is written into regions[r]->mycellgrid with
 *     tmpdefgseeds = identity, then the reference's own solve_REPLACE_CA_STRUCTURE
 *     (SCORE_Kernel.cpp:6353) maps it and counts cells;
 *   - orientations go into caHdl::myoripool, grains into mydefgpool/mydgoptimize,
 *     nuclei (orientation + site, rxg order) into myrxgpool.
 *
 * Modes:
 *   loop  : replays caHdl::solve_RXGROWTH (SCORE_Kernel.cpp:6497-6792) step for step,
 *           calling the reference's own region functions in the same order under the
 *           same OpenMP structure, minus the observation-only logging
 *           (log_OUTPUT_Diehl/log_PERCOLATION/rendering/cout).  Records per step
 *           t, dt, Xcells, Sv, full-cell count, P_max, rho_max at full precision and
 *           the final labels by the reference's clarify rule
 *           (SCORE_Io_Characterization.cpp:925-1000).  Also times the growth phases.
 *           With SCORE_LOG_AREA=<threshold> set it also takes the reference's on-the-fly
 *           grain-evolution log where log_OUTPUT_Diehl would (SCORE_OnTheFlyCharacterization.cpp:
 *           635-650: at the SingleGrainVolOverTime X logpoints, after the master block's
 *           counts): the reference's own log_grainevo and its RX area profile
 *           log_rxareaprofile(threshold) (:274-384; the log_rxareaprofile2 that
 *           log_OUTPUT_Diehl calls indexes an empty vector when rendering is off and
 *           advances the wrong loop counter, :423-427).  With SCORE_REDISCR="<nslots> <tmax>"
 *           it then evaluates the reference's caHdl::get_interpCellCount
 *           (SCORE_SolitaryUnitAveraging.cpp:1304-1365) for every grain at the ensemble's
 *           rediscretized times (postprocess_initrediscrtimes, :50-80).
 *           With SCORE_PERC=1 it ends with the reference's percolation analysis of the final
 *           state (log_PERCOLATION, SCORE_OnTheFlyCharacterization.cpp:777-875: the binarized
 *           structure of binarize_partiallyrxed_microstructure, then percAnalyzer's
 *           Hoshen-Kopelman labeling, compactify, checkLabeling, percolates and the sorted
 *           cluster-size distribution, SCORE_PercAnalyzer.cpp:118-665).
 *   asis  : calls the unmodified caHdl::solve_RXGROWTH and records t_end, step_end
 *           and the per-grain cell counts; used to prove `loop` is faithful.
 *   ptab  : dumps P(rxg,defg) from caregionMemHdl::reg_calc_mobilityweight
 *           (SCORE_Kernel.cpp:2460) and caHdl::calc_mobilityweight
 *           (SCORE_GrainBoundaryPhysics.cpp:50) for every pair.
 *
 * usage: score_ref_driver <mode> <params.uds> <domain.scdm> <outprefix>
 */
#include "SCORE_Kernel.h"

#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include <string>
#include <cstdlib>
#include <sstream>

/* grain-evolution logging of the loop mode (SCORE_LOG_AREA), off when < 0 */
static long g_log_area = -1;

struct Domain {
    uint32_t nx = 0, ny = 0, nz = 0, ndefg = 0, nrxg = 0;
    std::vector<uint32_t> grid;
    std::vector<double> defg;   // ndefg x (q0,q1,q2,q3,rho0)
    std::vector<double> rxgq;   // nrxg x (q0,q1,q2,q3)
    std::vector<uint32_t> site; // nrxg
    std::vector<double> tincub; // nrxg
};

static bool read_domain(const char* fn, Domain& d) {
    FILE* f = fopen(fn, "rb");
    if (!f) return false;
    char magic[4];
    uint32_t hdr[6];
    bool ok = fread(magic, 1, 4, f) == 4 && memcmp(magic, "SCDM", 4) == 0 && fread(hdr, 4, 6, f) == 6;
    if (ok) {
        d.nx = hdr[1]; d.ny = hdr[2]; d.nz = hdr[3]; d.ndefg = hdr[4]; d.nrxg = hdr[5];
        size_t n = (size_t)d.nx * d.ny * d.nz;
        d.grid.resize(n); d.defg.resize((size_t)d.ndefg * 5); d.rxgq.resize((size_t)d.nrxg * 4);
        d.site.resize(d.nrxg); d.tincub.resize(d.nrxg);
        ok = fread(d.grid.data(), 4, n, f) == n && fread(d.defg.data(), 8, d.defg.size(), f) == d.defg.size() &&
             fread(d.rxgq.data(), 8, d.rxgq.size(), f) == d.rxgq.size() &&
             fread(d.site.data(), 4, d.nrxg, f) == d.nrxg && fread(d.tincub.data(), 8, d.nrxg, f) == d.nrxg;
    }
    fclose(f);
    return ok;
}

static void push_ori(caHdl* ca, const double* q) {
    struct ori o;
    o.q0 = q[0]; o.q1 = q[1]; o.q2 = q[2]; o.q3 = q[3];
    o.closestideal = 0;  // counted as "random" texture class; not used by growth
    ca->myoripool.push_back(o);
}

/* Build an ensemble + one caHdl exactly as SIMULATE_myCAs does, then inject the domain. */
static caHdl* setup(const char* uds, const Domain& d) {
    ensembleHdl* ens = new ensembleHdl;
    if (!ens->open(READ, uds, &(ens->score_input))) { fprintf(stderr, "cannot open %s\n", uds); return NULL; }
    ens->myRank = 0; ens->nRanks = 1; ens->simid = 0;
    ens->init_ensprng(false);
    if (!ens->init_parameter()) fprintf(stderr, "WARNING: reference parameter validation reported a problem\n");

    caHdl* ca = new caHdl;
    ca->myensHdl = ens; ca->jobid = 0; ca->myensRank = 0; ca->nRanks = 1; ca->renderingForThisCA = false;
    ca->solve_INITIALIZATION();
    if (ca->myCAGeometry.nboxedge_rd != d.nx || ca->myCAGeometry.nboxedge_td != d.ny || ca->myCAGeometry.nboxedge_nd != d.nz) {
        fprintf(stderr, "geometry in .uds does not match domain file\n"); return NULL;
    }
    ca->solve_INITIALIZATION_THREADED_DOMAIN_DECOMPOSITION();

    for (uint32_t g = 0; g < d.ndefg; ++g) push_ori(ca, &d.defg[(size_t)g * 5]);
    for (uint32_t r = 0; r < d.nrxg; ++r) push_ori(ca, &d.rxgq[(size_t)r * 4]);
    for (uint32_t g = 0; g < d.ndefg; ++g) {
        struct cadefg dg;
        dg.worlddefgid = g; dg.caori = g; dg.cellcount = 0;
        dg.rho0 = d.defg[(size_t)g * 5 + 4]; dg.rho = dg.rho0;
        ca->mydefgpool.push_back(dg);
        struct dgopt op; op.rho = dg.rho0; op.id = g; op.cnt = 0;
        ca->mydgoptimize.push_back(op);
    }
    for (uint32_t r = 0; r < d.nrxg; ++r) {
        struct carxg rg;
        rg.caori = d.ndefg + r; rg.cellcount = 0; rg.nucsite = d.site[r]; rg.startingsite = d.site[r];
        rg.tincub = d.tincub[r];
        ca->myrxgpool.push_back(rg);
    }
    ca->ndefgseeds = d.ndefg;
    ca->tmpdefgseeds = new struct defgseed[d.ndefg];
    for (uint32_t g = 0; g < d.ndefg; ++g) { ca->tmpdefgseeds[g].mydefgpoolid = g; ca->tmpdefgseeds[g].ensdefgpoolid = g; }

    const uint32_t nx = d.nx, nxy = d.nx * d.ny;
    for (size_t r = 0; r < ca->regions.size(); ++r) {
        caregionMemHdl* re = ca->regions[r];
        uint32_t c = 0;
        for (uint32_t z = re->myGeom.nreg_ndmin; z <= re->myGeom.nreg_ndmax; ++z)
            for (uint32_t y = re->myGeom.nreg_tdmin; y <= re->myGeom.nreg_tdmax; ++y)
                for (uint32_t x = re->myGeom.nreg_rdmin; x <= re->myGeom.nreg_rdmax; ++x)
                    re->mycellgrid[c++] = d.grid[(size_t)x + (size_t)y * nx + (size_t)z * nxy];
        re->reg_nmydefgpool = d.ndefg;
    }
    ca->nmydefgpool = d.ndefg;
    ca->solve_REPLACE_CA_STRUCTURE();
    return ca;
}

struct StepRec {
    uint32_t step, pad;
    double t, dt, Xcells;
    uint64_t Sv, nfull;
    double Pmax, rhomax, dXstep;
};

/* Replay of caHdl::solve_RXGROWTH (SCORE_Kernel.cpp:6497-6792) minus observation-only logging. */
static int run_loop(caHdl* ca, std::vector<StepRec>& rec, double phase_s[5], double& loop_s) {
    ca->t = 0.0; ca->X = 0.0; ca->Xcells = 0.0; ca->dXstep = 0.0; ca->Sv = 0; ca->step = 0;
    ca->log_initialization();
    ca->update_mydgoptimize_rho();
    ca->update_mydgoptimize_cnt();
    ca->update_myrhomax();
    ca->update_temperature();
    ca->update_atomisticproperties();
    ca->update_intrinsicmobilities();
    ca->dt = ca->get_dtmax_minimum();
    { StepRec r0; memset(&r0, 0, sizeof r0); r0.dt = ca->dt; r0.rhomax = ca->myrhomax; rec.push_back(r0); }

    double tgrow = 0, tupd = 0, tsync = 0, tdefrag = 0;
    double t0loop = 0;
    #pragma omp parallel
    {
        int tid = omp_get_thread_num();
        caregionMemHdl* me = ca->regions[tid];
        me->ompshar_init_myRXFrontInside();
        me->ompshar_init_myRXFrontBorder();
        #pragma omp barrier
        vector<rxgcommit>* sync = new vector<rxgcommit>;
        ca->ompshar_sim_myCA_sitesaturatedNucleation(sync);
        #pragma omp barrier
        #pragma omp critical
        {
            for (uint32_t s = 0; s < sync->size(); s++) {
                ca->myrxgpool[sync->at(s).nrxgid].nucsite = sync->at(s).nucsite;
                ca->myrxgpool[sync->at(s).nrxgid].tincub = sync->at(s).tincub;
            }
        }
        delete sync;
        #pragma omp barrier
        #pragma omp master
        {
            for (uint32_t r = 0; r < ca->regions.size(); r++) {
                if (ca->regions[r]->reg_myMobilityWeightMax >= ca->myMobilityWeightMax) ca->myMobilityWeightMax = ca->regions[r]->reg_myMobilityWeightMax;
                ca->nmynuclei = ca->nmynuclei + ca->regions[r]->reg_nmynuclei;
            }
            rec[0].Pmax = ca->myMobilityWeightMax;
            t0loop = omp_get_wtime();
        }
        #pragma omp barrier
        for (uint32_t it = 0; it < DEFAULT_NMAX; it++) {
            bool operative = !((ca->Xcells >= ca->myCAGeometry.nboxvol_rdtdnd) || (ca->X > ca->XMAX) || (it > ca->NTSTEPSMAX) ||
                               (ca->t > ca->tprocessingend) || (ca->t > ca->TMAX));
            if (!operative) break;  /* every thread sees the same shared state */
            if (ca->onthefly_defragmentation == true) {
                if (me->reg_defrag_cnt < ca->defragRXFront_atthisX.size() && ca->Xcells >= ca->defragRXFront_atthisX[me->reg_defrag_cnt]) {
                    me->ompshar_defragmentation();
                    me->reg_defrag_cnt++;
                }
            }
            me->ompshar_sim_myCA_calcGrowthStepInside();
            me->ompshar_sim_myCA_calcGrowthStepBorder();
            me->ompshar_sim_myCA_updateFullRXInside();
            me->ompshar_clear_halo_bookkeeping();
            me->ompshar_sim_myCA_updateFullRXBorder();
            #pragma omp barrier
            me->ompshar_synchronize_haloregions_rx();
            #pragma omp barrier
            #pragma omp master
            {
                double gmax = 0, umax = 0, smax = 0, dmax = 0;
                for (size_t r = 0; r < ca->regions.size(); ++r) {
                    caregionMemHdl* q = ca->regions[r];
                    gmax = std::max(gmax, q->dtCalcGrowthInside + q->dtCalcGrowthBorder);
                    umax = std::max(umax, q->dtUpdateInside + q->dtUpdateBorder);
                    smax = std::max(smax, q->dtSyncHalo);
                    dmax = std::max(dmax, q->dtDefragment);
                    q->dtDefragment = 0.0;
                }
                tgrow += gmax; tupd += umax; tsync += smax; tdefrag += dmax;

                ca->dXstep = 0.0; ca->Sv = 0;
                double mymobmax = DEFAULT_PMAX;
                uint64_t nupd = 0;
                for (uint32_t r = 0; r < ca->regions.size(); r++) {
                    caregionMemHdl* q = ca->regions[r];
                    if (q->reg_myMobilityWeightMax >= mymobmax) mymobmax = q->reg_myMobilityWeightMax;
                    ca->dXstep = ca->dXstep + (q->reg_dXstepInside + q->reg_dXstepBorder);
                    ca->Sv = ca->Sv + (q->reg_SvInside + q->reg_SvBorder);
                    nupd += q->reg_nUpdatedCellsInside + q->reg_nUpdatedCellsBorder;
                    ca->Xcells = ca->Xcells + ((double)(q->reg_nUpdatedCellsInside + q->reg_nUpdatedCellsBorder));
                }
                ca->myMobilityWeightMax = mymobmax;
                ca->X = (ca->Xcells / ((double)ca->myCAGeometry.nboxvol_rdtdnd));
                ca->synchronize_myrxgpool_counts();
                ca->synchronize_mydefpool_counts();
                if (ca->myRecoveryModel.RecoveryConsider != RECOVERY_NO) ca->update_mydgoptimize_rho();
                ca->update_mydgoptimize_cnt();
                ca->update_myrhomax();
                /* log_OUTPUT_Diehl's grain-evolution branch (SCORE_OnTheFlyCharacterization.cpp:646-650),
                   bounds test first */
                if (g_log_area >= 0 && ca->loginfo_grainevo_cnt < ca->output_atthisX.size() &&
                    ca->Xcells >= ca->output_atthisX[ca->loginfo_grainevo_cnt]) {
                    ca->ompcrit_clarify_status_infectedcells(RXFRACTION_THRESHOLD);
                    ca->log_grainevo();
                    ca->log_rxareaprofile((uint32_t)g_log_area);
                }
                StepRec r;
                memset(&r, 0, sizeof r);
                r.Sv = ca->Sv; r.nfull = nupd; r.Xcells = ca->Xcells; r.Pmax = ca->myMobilityWeightMax;
                r.rhomax = ca->myrhomax; r.dXstep = ca->dXstep;
                ca->t += ca->dt;
                ca->update_temperature();
                ca->update_atomisticproperties();
                ca->update_microchemistry();
                ca->update_intrinsicmobilities();
                ca->update_deformedsubstructure();
                ca->dt = ca->get_dtmax_minimum();
                ca->step++;
                r.step = ca->step; r.t = ca->t; r.dt = ca->dt;
                rec.push_back(r);
            }
            #pragma omp barrier
        }
        #pragma omp master
        { loop_s = omp_get_wtime() - t0loop; }
    }
    ca->tsimend = ca->t;  /* as solve_RXGROWTH leaves them (SCORE_Kernel.cpp:6752-6753) */
    ca->stepsimend = ca->step;
    phase_s[0] = tgrow; phase_s[1] = tupd; phase_s[2] = tsync; phase_s[3] = tdefrag;
    phase_s[4] = tgrow + tupd + tsync + tdefrag;
    return 0;
}

/* Final labels by the reference's clarify rule (SCORE_Io_Characterization.cpp:925-1000). */
static void final_labels(caHdl* ca, const Domain& d, std::vector<uint32_t>& lab) {
    const uint32_t nx = d.nx, nxy = d.nx * d.ny;
    lab.assign((size_t)nx * d.ny * d.nz, 0xFFFFFFFFu);
    for (size_t r = 0; r < ca->regions.size(); ++r) {
        caregionMemHdl* re = ca->regions[r];
        uint32_t c = 0;
        for (uint32_t z = re->myGeom.nreg_ndmin; z <= re->myGeom.nreg_ndmax; ++z)
            for (uint32_t y = re->myGeom.nreg_tdmin; y <= re->myGeom.nreg_tdmax; ++y)
                for (uint32_t x = re->myGeom.nreg_rdmin; x <= re->myGeom.nreg_rdmax; ++x)
                    lab[(size_t)x + (size_t)y * nx + (size_t)z * nxy] = re->mycellgrid[c++];
    }
    ca->ompcrit_clarify_status_infectedcells(RXFRACTION_THRESHOLD);
    for (size_t r = 0; r < ca->cellStatii.size(); ++r) {
        if (!ca->cellStatii[r]) continue;
        for (size_t i = 0; i < ca->cellStatii[r]->size(); ++i) lab[ca->cellStatii[r]->at(i).ixyz] = ca->cellStatii[r]->at(i).gid;
    }
}

static bool write_file(const std::string& fn, const void* p, size_t bytes) {
    FILE* f = fopen(fn.c_str(), "wb");
    if (!f) return false;
    bool ok = fwrite(p, 1, bytes, f) == bytes;
    fclose(f);
    return ok;
}

int main(int argc, char** argv) {
    if (argc < 5) { fprintf(stderr, "usage: %s loop|asis|ptab params.uds domain.scdm outprefix\n", argv[0]); return 2; }
    std::string mode = argv[1], out = argv[4];
    if (const char* la = getenv("SCORE_LOG_AREA")) g_log_area = atol(la);
    Domain d;
    if (!read_domain(argv[3], d)) { fprintf(stderr, "cannot read domain %s\n", argv[3]); return 2; }
    std::streambuf* keep = std::cout.rdbuf();
    std::ofstream sink("/dev/null");
    std::cout.rdbuf(sink.rdbuf());  // the reference prints progress to cout; keep stdout clean
    caHdl* ca = setup(argv[2], d);
    if (!ca) { std::cout.rdbuf(keep); return 3; }

    if (mode == "ptab") {
        std::vector<double> reg((size_t)d.nrxg * d.ndefg), nuc((size_t)d.nrxg * d.ndefg);
        for (uint32_t r = 0; r < d.nrxg; ++r)
            for (uint32_t g = 0; g < d.ndefg; ++g) {
                reg[(size_t)r * d.ndefg + g] = ca->regions[0]->reg_calc_mobilityweight(r, g);
                nuc[(size_t)r * d.ndefg + g] = ca->calc_mobilityweight(r, g);
            }
        std::cout.rdbuf(keep);
        return (write_file(out + ".ptab", reg.data(), reg.size() * 8) && write_file(out + ".ptabnuc", nuc.data(), nuc.size() * 8)) ? 0 : 4;
    }
    if (mode == "asis") {
        double w0 = omp_get_wtime();
        ca->solve_RXGROWTH();
        double w1 = omp_get_wtime();
        std::cout.rdbuf(keep);
        FILE* f = fopen((out + ".asis").c_str(), "w");
        fprintf(f, "t_end %a\nstep_end %u\nwall_s %.6f\nthreads %d\n", ca->tsimend, ca->stepsimend, w1 - w0, omp_get_max_threads());
        for (size_t r = 0; r < ca->myrxgpool.size(); ++r) fprintf(f, "rxg %zu %u\n", r, ca->myrxgpool[r].cellcount);
        for (size_t g = 0; g < ca->mydefgpool.size(); ++g) fprintf(f, "defg %zu %u\n", g, ca->mydefgpool[g].cellcount);
        fclose(f);
        return 0;
    }
    std::vector<StepRec> rec;
    double phase[5], loop_s = 0;
    run_loop(ca, rec, phase, loop_s);
    std::vector<uint32_t> lab;
    final_labels(ca, d, lab);
    std::cout.rdbuf(keep);
    uint64_t sumSv = 0;
    for (size_t i = 1; i < rec.size(); ++i) sumSv += rec[i].Sv;
    FILE* f = fopen((out + ".summary").c_str(), "w");
    fprintf(f, "steps %zu\nt_end %a\nsum_Sv %llu\nthreads %d\nloop_s %.6f\ngrow_s %.6f\nupdate_s %.6f\nsync_s %.6f\ndefrag_s %.6f\nphases_s %.6f\n",
            rec.size() - 1, ca->t, (unsigned long long)sumSv, omp_get_max_threads(), loop_s, phase[0], phase[1], phase[2], phase[3], phase[4]);
    for (size_t r = 0; r < ca->myrxgpool.size(); ++r) fprintf(f, "rxg %zu %u\n", r, ca->myrxgpool[r].cellcount);
    for (size_t g = 0; g < ca->mydefgpool.size(); ++g) fprintf(f, "defg %zu %u\n", g, ca->mydefgpool[g].cellcount);
    fclose(f);
    bool ok = write_file(out + ".trace", rec.data(), rec.size() * sizeof(StepRec)) &&
              write_file(out + ".labels", lab.data(), lab.size() * 4);
    if (ok && g_log_area >= 0) {
        /* grain evolution: per snapshot t, X (f64), step, Sv (u32), counts of every grain (u32, deformed then rx) */
        FILE* g = fopen((out + ".grainevo").c_str(), "wb");
        for (size_t i = 0; g && i < ca->mygrainevolution.size(); ++i) {
            const loginfo_grainevo_ca& e = ca->mygrainevolution[i];
            const uint32_t hdr[2] = {e.localtstep, e.localSv};
            fwrite(&e.localtime, 8, 1, g); fwrite(&e.localX, 8, 1, g); fwrite(hdr, 4, 2, g);
            fwrite(e.localdatabucket, 4, e.nlocaldata, g);
        }
        if (g) fclose(g);
        /* RX area profile: per snapshot t, X (f64), step, 0 (u32), then (rx, deformed) cells per z slice (u32) */
        FILE* a = fopen((out + ".rxprofile").c_str(), "wb");
        for (size_t i = 0; a && i < ca->myrxprofile.size(); ++i) {
            const loginfo_rxareaprofile_ca& e = ca->myrxprofile[i];
            const uint32_t hdr[2] = {e.localstep, 0u};
            fwrite(&e.localtime, 8, 1, a); fwrite(&e.localX, 8, 1, a); fwrite(hdr, 4, 2, a);
            fwrite(e.localdatabucket, 4, 2 * (size_t)d.nz, a);
        }
        if (a) fclose(a);
        ok = g && a;
    }
    if (ok && getenv("SCORE_PERC") && d.nx == d.ny && d.nx == d.nz) {
        /* percolation record: n clusters, largest cluster, percolates, checkLabeling failed (u32), the sorted cluster sizes (u32),
           then the binarized structure (one byte per cell) */
        std::vector<bool>* bin = new std::vector<bool>;
        ca->binarize_partiallyrxed_microstructure(bin);
        std::vector<uint8_t> bytes(bin->size());
        for (size_t i = 0; i < bin->size(); ++i) bytes[i] = (*bin)[i] ? 1 : 0;
        percAnalyzer* hk = new percAnalyzer;
        hk->initialize(bin, d.nx);
        delete bin;
        std::cout.rdbuf(sink.rdbuf());
        hk->hoshen_kopelman();
        hk->compactify();
        std::ostringstream cerr_text;  /* checkLabeling reports a cell whose neighbour carries another label on cerr */
        std::streambuf* keep_err = std::cerr.rdbuf(cerr_text.rdbuf());
        hk->checkLabeling();
        std::cerr.rdbuf(keep_err);
        const bool perc = hk->percolates();
        hk->determine_clustersize_distr();
        std::cout.rdbuf(keep);
        const uint32_t split = cerr_text.str().find("failed assertion") != std::string::npos ? 1u : 0u;
        const uint32_t hdr[4] = {hk->getNCluster(), hk->getClusterSize(), perc ? 1u : 0u, split};
        std::vector<uint32_t> dist(hdr[0]);
        if (hdr[0]) hk->handover_distribution(dist.data());
        delete hk;
        FILE* f = fopen((out + ".perc").c_str(), "wb");
        ok = f && fwrite(hdr, 4, 4, f) == 4 && fwrite(dist.data(), 4, dist.size(), f) == dist.size() &&
             fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
        if (f) fclose(f);
    }
    const char* rd = getenv("SCORE_REDISCR");
    if (ok && rd) {
        /* postprocess_initrediscrtimes (SCORE_SolitaryUnitAveraging.cpp:62-80) with tensmin = 0, then
           get_interpCellCount of every grain at every rediscretized time (doubles, [slot][grain]) */
        unsigned nslots = 0;
        double tmax = 0.0;
        if (sscanf(rd, "%u %lf", &nslots, &tmax) != 2 || nslots < 2) return 5;
        const double ttmin = 0.0, dt = (tmax - ttmin) / ((double)(nslots - 1));
        const uint32_t ng = (uint32_t)(ca->mydefgpool.size() + ca->myrxgpool.size());
        std::vector<double> v((size_t)nslots * ng);
        for (uint32_t n = 0; n < nslots; ++n) {
            const double when = ttmin + ((double)(n + 1) * dt);
            for (uint32_t id = 0; id < ng; ++id) v[(size_t)n * ng + id] = ca->get_interpCellCount(id, when);
        }
        ok = write_file(out + ".interp", v.data(), v.size() * 8);
    }
    return ok ? 0 : 4;
}
