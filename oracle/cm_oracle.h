/* Test infrastructure only (the oracle): a plain-C, FP64 restatement of the reference
 * cell-model update for ten Tusscher-Panfilov 2006, Courtemanche 1998, O'Hara-Rudy 2011
 * (the reference's variant: Passini/Dutta I_Na gates, troponin, SAC) and Tomek 2019, used by the
 * tests as the checker and by bench.py as the timed CPU baseline. The product never
 * links or calls it.
 *
 * State blocks use the reference's backup layout (GetBase()/GetSize()):
 *   TT2 (36 doubles, TenTusscher2.h:77-123):  Ca_i CaSR CaSS Na_i K_i Array[18] m h j xr1 xr2 xs r s d f f2 fCa Rq
 *   CRN (22 doubles, CourtemancheEtAl.h:32-42): Ca_i Ca_up Ca_rel h j oi ui Xr Xs u v w Na_i K_i m oa ua d f f_Ca I_SAC Ca_TRPN
 *   ORd (59 doubles, OHaraRudy.h:31-52): 42 states from m to Ca_TRPN (h_CaMK_fast unused), then
 *        I_Na_fast I_Na_late I_to I_CaL I_CaNa I_CaK I_Kr I_Ks I_K1 I_NaCa_i I_NaCa_ss I_NaK I_Nab I_Cab I_Kb I_pCa I_SAC
 *   Tomek (84 doubles, Tomek.h:33-52): 48 states from m to Ca_TRPN, then 36 stored currents and fluxes
 *
 * Parameter vectors P are indexed by this file's own parameter lists (names as in the
 * reference .ev files); derived quantities are recomputed here (restating
 * TenTusscher2Parameters::Calculate and CourtemancheParameters::Calculate).
 */
#ifndef CM_ORACLE_H
#define CM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { CMO_TT2 = 0, CMO_CRN = 1, CMO_ORD = 2, CMO_TOM = 3 };
enum { CMO_RTDT = 4000 };

int cmo_n_params(int model);
const char *cmo_param_name(int model, int i);
int cmo_param_index(int model, const char *name);
int cmo_state_doubles(int model);
int cmo_n_tables(int model);
const char *cmo_table_name(int model, int k);

/* Fills the derived slots of P (the tail of the parameter list) from the base ones. */
void cmo_derive(int model, double *P);

/* tables: cmo_n_tables(model) * CMO_RTDT doubles, table k at tables + k*CMO_RTDT. */
int cmo_build_tables(int model, const double *P, double dt, double *tables);
void cmo_init_state(int model, const double *P, double *block);
double cmo_init_vm(int model, const double *P);

/* One reference Calc: returns dV [V], updates block in place. dt [s], V [V]. */
double cmo_calc(int model, const double *P, const double *tables, double *block, double dt, double V,
                double i_ext, double stretch);

/* Driver loop over cells (CellModel.h:405-420): n_steps of Vm += Calc(dt, Vm, i_ext(t), 1, 1).
 * het_idx[k] names parameter slot k overridden per cell by het_vals[k*n_cells + c].
 * trace (optional): Vm before every rec_every-th step, trace[c*n_rec + s/rec_every].
 * textbegin may be per cell (textbegin_per_cell != NULL) or one value for all. */
int cmo_run(int model, const double *P, const double *tables, long n_cells, double *blocks, double *Vm,
            int n_het, const int *het_idx, const double *het_vals, long n_steps, double dt, double t0,
            double textbegin, const double *textbegin_per_cell, double textlen, double bcl, double amp,
            long rec_every, double *trace, int n_threads);

/* Explicit monodomain steps (acCELLerate::IntraStep, Godunov): per step B = A*Vm (CSR, row
 * entries summed in order), i_ext = B*scale + stimulus, Vm += Calc(dt, Vm, i_ext, 1, 1), then
 * activation times (act[c] = t where act[c] == -1 and the new Vm >= act_threshold). scale NULL:
 * uniform_scale. trace (optional): Vm before every rec_every-th step. Returns -3 when a Vm became
 * NaN or left +-vm_range (vm_range > 0). */
int cmo_mono_run(int model, const double *P, const double *tables, long n_cells, double *blocks, double *Vm,
                 int n_het, const int *het_idx, const double *het_vals, const long *rowptr, const int *col,
                 const double *val, const double *scale, double uniform_scale, long n_steps, double dt, double t0,
                 double textbegin, const double *textbegin_per_cell, double textlen, double bcl, double amp,
                 double *act, double act_threshold, double vm_range, long rec_every, double *trace, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
