// Driver that runs the reference DMD sources (src_v4.5.7, compiled unmodified against the shims in
// oracle/ref_shim) on a directory holding param.in and ldbd_data/. Test infrastructure only: it
// produces the golden vectors that pin the oracle and the GPU path.
//
// It defines the globals of main.cpp:2-8 and re-creates dm_dynamics_jdftx (main.cpp:38-74), then
// runs one of these modes in the current directory:
//   dump  OUT            setup arrays after construction (e_dm, f_dm, initial dm, H_BS, folded P)
//   rhs   IN OUT         for each (t, y) record of IN: func(t,y,dydt) (DensityMatrix_Dynamics.h:358),
//                        electronphonon::evolve_driver (evolve_eph.cpp:21) and
//                        singdenmat_k::evolve_coh (DenMat.cpp:29) on the same y
//   rk4   DT_FS N EVERY OUT  classic fixed-step RK4 calling DMD's own func; S_z is measured with
//                        DMD's observable (observable.h:113) every EVERY steps
//   gsl                  DMD's native evolve_gsl (RKF45 through the GSL restatement)
//   euler                DMD's native evolve_euler
//   tau                  compute(t0) + report_tau(0) (DensityMatrix_Dynamics.h:75)
//   pee   IN OUT         e-e model: for each (t, y) record of IN, electronphonon::reset_scatt
//                        (ElectronPhonon.cpp:15-42) on that density matrix -- the screening update
//                        and P = P_eph (+ P_eimp) + scale_ee P_ee(rho) (ElecElec_Model.h:186-262) --
//                        then the folded P1, P2 and the screening density
#include "DensityMatrix_Dynamics.h"
#include <vector>

bool DEBUG = false;
string dir_debug = "debug_info/";
bool ionode = false;
algorithm alg;
string code = "";
string material_model = "";
ODEparameters ode;

typedef dm_dynamics<lattice, electron, electronlight, electronphonon> dyn_t;

static void write_bin(const std::string& path, const void* p, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
  if (bytes) fwrite(p, 1, bytes, f);
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc < 2) { fprintf(stderr, "usage: dmd_ref dump|rhs|rk4|gsl|euler|tau ...\n"); return 2; }
  std::string mode = argv[1];

  // main.cpp:18-28
  mpkpair.mpi_init(); mpkpair2.mpi_init(); mpk.mpi_init(); mpk_morek.mpi_init();
  ionode = mpkpair.ionode;
  parameters* param = new parameters();
  param->read_param();
  init_model(param);
  if (material_model != "none") { fprintf(stderr, "only material_model = none is supported\n"); return 2; }

  // main.cpp:38-74
  lattice* latt = new lattice(param);
  electron* elec = new electron(&mpk, &mpk_morek, latt, param);
  mpk.distribute_var("dm_dynamics_driver", elec->nk);
  if (elec->nk_morek > 0) mpk_morek.distribute_var("dm_dynamics_driver", elec->nk_morek);
  param->mu = elec->set_mu_and_n(param->carrier_density);
  elec->compute_b2(param->de_measure, param->degauss_measure, param->degthr);
  elec->compute_Bin2();
  elec->compute_dm_Bpert_1st(param->Bpert, param->t0);
  if (elec->B.length() > 1e-10 || alg.read_Bso) elec->set_H_BS(mpk.varstart, mpk.varend);
  if (abs(elec->scale_Ez) > 1e-10) elec->set_H_Ez(mpk.varstart, mpk.varend);
  phonon* ph = new phonon(latt, param, elec);
  electronlight* elight = nullptr;
  if (pmp.active()) { fprintf(stderr, "laser is not supported by this driver\n"); return 2; }
  electronphonon* eph = new electronphonon(&mpkpair, latt, param, elec, ph, alg.eph_sepr_eh, !alg.eph_need_elec);
  if (alg.scatt_enable) mpkpair.distribute_var("dm_dynamics_jdftx", eph->nkpair_glob);
  if (alg.scatt_enable) eph->set_eph();
  if (alg.scatt_enable && alg.linearize && param->need_imsig) eph->compute_imsig();
  if (alg.scatt_enable) eph->analyse_g2(param->de_measure, param->degauss_measure, param->degthr);
  if (alg.scatt_enable) eph->analyse_g2_ei(param->de_measure, param->degauss_measure, param->degthr);
  dyn_t* dmdyn = new dyn_t(latt, param, elec, elight, eph);

  const int nk = elec->nk, nbdm = elec->nb_dm;
  const size_t n = (size_t)nk * nbdm * nbdm;

  if (mode == "dump") {
    std::string out = argv[2];
    FILE* m = fopen((out + "/meta.txt").c_str(), "w");
    fprintf(m, "nk %d\nnb_dm %d\nbstart %d\nbend %d\nnkpair %d\nprefac_eph %.17g\nnk_full %.17g\nt0 %.17g\n"
               "temperature %.17g\nmu %.17g\ncell_size %.17g\ncell_size_cmd %.17g\nhas_H %d\n",
            nk, nbdm, eph->bStart, eph->bEnd, eph->nkpair_glob, eph->prefac_eph, elec->nk_full, param->t0,
            param->temperature, param->mu, latt->cell_size, latt->cell_size_cmd, dmdyn->sdmk->Hcoh ? 1 : 0);
    fprintf(m, "nv_dm %d\nmue %.17g\nmuh %.17g\nddmdteq %d\nlinearize %d\n", elec->nv_dm, dmdyn->sdmk->mue,
            dmdyn->sdmk->muh, alg.ddmdteq ? 1 : 0, alg.linearize ? 1 : 0);
    if (eph->ee_model) {  // e-e model constants (ElecElec_Model.h:22-37, Coulomb_Model.h:415-423, 555-569)
      coulomb_model* cm = eph->coul_model;
      fprintf(m, "ee 1\nee_nfree %.17g\nee_scale %.17g\nee_degauss %.17g\nee_ethr %.17g\nee_eps %.17g\n"
                 "ee_meff %.17g\nee_T %.17g\nee_nv %d\nee_antisym %d\nee_qscr2_debye %.17g\nee_nbw %d\n",
              clp.nfreetot, eph->scale_ee, eph->ee_model->degauss, eph->ee_model->ethr, clp.eps, clp.meff, cm->T,
              cm->nv, eep.antisymmetry ? 1 : 0, cm->qscr2_debye, elec->nb_wannier);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) fprintf(m, "ee_ggt%d%d %.17g\n", i, j, latt->GGT(i, j));
    }
    fclose(m);
    if (alg.ddmdteq || alg.linearize) write_bin(out + "/f_eq.bin", dmdyn->sdmk->f_eq[0], sizeof(double) * nk * nbdm);
    if (alg.ddmdteq) write_bin(out + "/ddmdt_eq.bin", eph->ddmdt_eq[0], sizeof(complex) * nk * eph->nb * eph->nb);
    write_bin(out + "/e_dm.bin", elec->e_dm[0], sizeof(double) * nk * nbdm);
    write_bin(out + "/f_dm.bin", elec->f_dm[0], sizeof(double) * nk * nbdm);
    write_bin(out + "/dm0.bin", dmdyn->sdmk->dm[0], sizeof(complex) * n);
    if (dmdyn->sdmk->Hcoh) write_bin(out + "/Hcoh.bin", dmdyn->sdmk->Hcoh[0], sizeof(complex) * n);
    size_t np4 = (size_t)eph->nkpair_proc * (size_t)std::pow(eph->nb, 4);
    if (alg.linearize) {  // the linear operators replace P1, P2 (ElectronPhonon_linear.cpp:3-31)
      write_bin(out + "/Lscij.bin", eph->Lscij[0], sizeof(complex) * np4);
      write_bin(out + "/Lscji.bin", eph->Lscji[0], sizeof(complex) * np4);
    } else {
      write_bin(out + "/P1.bin", eph->P1[0], sizeof(complex) * np4);
      write_bin(out + "/P2.bin", eph->P2[0], sizeof(complex) * np4);
    }
    return 0;
  }
  if (mode == "rhs") {
    FILE* in = fopen(argv[2], "rb");
    std::string out = argv[3];
    if (!in) { fprintf(stderr, "cannot read %s\n", argv[2]); return 2; }
    std::vector<double> y(2 * n), dydt(2 * n);
    complex** tmp = alloc_array(nk, nbdm * nbdm);
    complex** tmp1 = alloc_array(nk, nbdm * nbdm);
    std::vector<double> all_f, all_eph, all_coh;
    double t;
    while (fread(&t, sizeof(double), 1, in) == 1) {
      if (fread(y.data(), sizeof(double), 2 * n, in) != 2 * n) { fprintf(stderr, "short record\n"); return 2; }
      func<lattice, electron, electronlight, electronphonon>(t, y.data(), dydt.data(), dmdyn);
      all_f.insert(all_f.end(), dydt.begin(), dydt.end());
      // the scattering and coherent parts on the same state (compute() order: 1-dm, coh, eph)
      copy_complex_from_real(dmdyn->sdmk->dm, y.data(), n);
      dmdyn->sdmk->set_oneminusdm();
      eph->evolve_driver(t, dmdyn->sdmk->dm, dmdyn->sdmk->oneminusdm, tmp);
      all_eph.insert(all_eph.end(), (double*)tmp[0], (double*)tmp[0] + 2 * n);
      if (dmdyn->sdmk->Hcoh) dmdyn->sdmk->evolve_coh(t, tmp1);
      else zeros(tmp1, nk, nbdm * nbdm);
      all_coh.insert(all_coh.end(), (double*)tmp1[0], (double*)tmp1[0] + 2 * n);
    }
    fclose(in);
    write_bin(out + "/dydt.bin", all_f.data(), all_f.size() * sizeof(double));
    write_bin(out + "/ddmdt_eph.bin", all_eph.data(), all_eph.size() * sizeof(double));
    write_bin(out + "/ddmdt_coh.bin", all_coh.data(), all_coh.size() * sizeof(double));
    return 0;
  }
  if (mode == "rk4") {
    const double h = atof(argv[2]) * fs;
    const long nsteps = atol(argv[3]), every = atol(argv[4]);
    std::string out = argv[5];
    std::vector<double> y(2 * n), k1(2 * n), k2(2 * n), k3(2 * n), k4(2 * n), yt(2 * n);
    copy_real_from_complex(y.data(), dmdyn->sdmk->dm, n);
    const double t0 = dmdyn->sdmk->t;
    const double hh = 0.5 * h, h6 = h / 6.0;
    for (long s = 0; s < nsteps; ++s) {
      const double t = t0 + (double)s * h;
      auto f = func<lattice, electron, electronlight, electronphonon>;
      f(t, y.data(), k1.data(), dmdyn);
      for (size_t i = 0; i < 2 * n; ++i) yt[i] = y[i] + hh * k1[i];
      f(t + hh, yt.data(), k2.data(), dmdyn);
      for (size_t i = 0; i < 2 * n; ++i) yt[i] = y[i] + hh * k2[i];
      f(t + hh, yt.data(), k3.data(), dmdyn);
      for (size_t i = 0; i < 2 * n; ++i) yt[i] = y[i] + h * k3[i];
      f(t + h, yt.data(), k4.data(), dmdyn);
      for (size_t i = 0; i < 2 * n; ++i) y[i] = y[i] + h6 * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
      if ((s + 1) % every == 0) {
        const double t1 = t0 + (double)(s + 1) * h;
        copy_complex_from_real(dmdyn->sdmk->dm, y.data(), n);
        dmdyn->sdmk->t = t1;
        dmdyn->ob->measure("sz", "", true, false, t1, dmdyn->sdmk->dm);
      }
    }
    write_bin(out + "/y_final.bin", y.data(), y.size() * sizeof(double));
    return 0;
  }
  if (mode == "pee") {
    FILE* in = fopen(argv[2], "rb");
    std::string out = argv[3];
    if (!in || !eph->ee_model) { fprintf(stderr, "pee needs %s and an e-e model\n", argv[2]); return 2; }
    std::vector<double> y(2 * n);
    std::vector<complex> all1, all2;
    std::vector<double> nfree;
    const size_t np4 = (size_t)eph->nkpair_proc * (size_t)std::pow(eph->nb, 4);
    double t;
    while (fread(&t, sizeof(double), 1, in) == 1) {
      if (fread(y.data(), sizeof(double), 2 * n, in) != 2 * n) { fprintf(stderr, "short record\n"); return 2; }
      copy_complex_from_real(dmdyn->sdmk->dm, y.data(), n);
      dmdyn->sdmk->set_oneminusdm();
      eph->reset_scatt(false, true, dmdyn->sdmk->dm, dmdyn->sdmk->oneminusdm, t, dmdyn->sdmk->f_eq);
      all1.insert(all1.end(), eph->P1[0], eph->P1[0] + np4);
      all2.insert(all2.end(), eph->P2[0], eph->P2[0] + np4);
      nfree.push_back(clp.nfreetot);
    }
    fclose(in);
    write_bin(out + "/pee_P1.bin", all1.data(), all1.size() * sizeof(complex));
    write_bin(out + "/pee_P2.bin", all2.data(), all2.size() * sizeof(complex));
    write_bin(out + "/pee_nfree.bin", nfree.data(), nfree.size() * sizeof(double));
    return 0;
  }
  if (mode == "gsl") { dmdyn->evolve_gsl(); return 0; }
  if (mode == "euler") { dmdyn->evolve_euler(); return 0; }
  if (mode == "tau") { dmdyn->compute(dmdyn->sdmk->t); dmdyn->report_tau(0); return 0; }
  fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
