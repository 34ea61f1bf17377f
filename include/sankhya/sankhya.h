/*
 * sankhya.h -- public C API (handles + error codes) of the LP engine.
 * Signatures and error codes are those of the reference's
 * include/sankhya/sankhya.h:8-41. Behaviour differs where the reference was a
 * stub: sankhya_load_model reads MPS files (the name "fixture" still builds the
 * reference's built-in two-row LP, src/api/c_api.cpp:41-69), and sankhya_solve
 * runs the device Mehrotra IPM instead of the CPU primal simplex
 * (src/api/c_api.cpp:76-93). sankhya_get_solution is an addition.
 */
#ifndef SANKHYA_C_API_H
#define SANKHYA_C_API_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sankhya_env_s sankhya_env_t;
typedef struct sankhya_model_s sankhya_model_t;

#define SANKHYA_SUCCESS 0
#define SANKHYA_ERROR_INVALID_ARGUMENT 1
#define SANKHYA_ERROR_LOAD_FAILED 2
#define SANKHYA_ERROR_SOLVE_FAILED 3
#define SANKHYA_ERROR_NOT_AVAILABLE 4
#define SANKHYA_ERROR_INTERNAL 5

int sankhya_create_env(sankhya_env_t** env);
int sankhya_load_model(sankhya_env_t* env, const char* filename, sankhya_model_t** model);
int sankhya_solve(sankhya_model_t* model);
int sankhya_get_objval(sankhya_model_t* model, double* objval);
/* x (n) and pi (m) of the last successful solve; either may be NULL. */
int sankhya_get_solution(sankhya_model_t* model, double* x, double* pi, int* n, int* m);
void sankhya_free_model(sankhya_model_t* model);
void sankhya_free_env(sankhya_env_t* env);

#ifdef __cplusplus
}
#endif

#endif /* SANKHYA_C_API_H */
