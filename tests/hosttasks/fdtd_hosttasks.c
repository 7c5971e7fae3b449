/*
 * fdtd_hosttasks.c -- TEST INFRASTRUCTURE: host tasks for the reference FDTD graph, the counterpart
 * of the reference's HostTasks library (HostTasks/HostTasks.def exports host entry points with the
 * LPFNHOSTTASK signature of ptask/hosttask.h:28-31).  Each entry point runs one per-field task
 * (graphfdtd.cpp:185-312) through the oracle, so that the same graph can run with every task on the
 * host, every task on the GPU, or a mix, and the results be compared.
 *
 * Arguments (formal-parameter order of graphfdtd.cpp:398-436): in0, in1, in2, &FDTD_PARAMS, out.
 */
struct oracle_params;
int oracle_field_task_f32(int f, const float *a, const float *b, const float *c, const struct oracle_params *p,
                          float *out);

static void run(int f, unsigned n, void **a)
{
    if (n == 5)
        oracle_field_task_f32(f, (const float *)a[0], (const float *)a[1], (const float *)a[2],
                              (const struct oracle_params *)a[3], (float *)a[4]);
}

void HxComputation(unsigned n, void **a) { run(0, n, a); }
void HyComputation(unsigned n, void **a) { run(1, n, a); }
void HzComputation(unsigned n, void **a) { run(2, n, a); }
void ExComputation(unsigned n, void **a) { run(3, n, a); }
void EyComputation(unsigned n, void **a) { run(4, n, a); }
void EzComputation(unsigned n, void **a) { run(5, n, a); }
