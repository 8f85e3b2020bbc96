/*
 * fastcall.c -- CPython fast path for the per-move drop-in calls.
 *
 * fullrmc's PairDistributionConstraint calls multiple_pairs_histograms_coords
 * and full_pairs_histograms_coords four times per move, and the Engine
 * transforms the moved coordinates (PairDistributionConstraints.py:1044-1129,
 * Engine.py:3222-3223).  Their Python wrappers (fullrmc_gb300.pairs_histograms,
 * .boundary_conditions_collection) spend tens of microseconds per call in
 * ctypes pointer objects and argument coercion.  This module does the same
 * work for the common case -- C-contiguous numpy arrays of the right dtype
 * and rank, plain scalars -- and calls the C ABI of libfrmc_gpu.so directly.
 *
 * Each function returns None when an argument is anything else (a list, a
 * non-contiguous array, a float where an integer is expected, ...): the
 * Python wrapper then runs its full argument checks, which raise the
 * exceptions fullrmc's Cython modules raise.  A library error comes back as
 * the integer status, which the wrapper turns into its exception.  The GPU
 * work and its results are those of the wrappers' own calls.
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <stdint.h>

#include "frmc_gpu.h"

static PyObject *g_ndarray;  /* numpy.ndarray */
static PyObject *g_floating; /* numpy.floating */
static PyObject *g_zeros;    /* numpy.zeros */
static PyObject *g_float32;  /* numpy.float32 */

/* A C-contiguous ndarray with `ndim` dimensions of 4-byte items of format
 * `fmt` ('f' float32, 'i' int32); 0 (and nothing held) otherwise. */
static int take(PyObject *o, Py_buffer *v, char fmt, int ndim)
{
    if (PyObject_IsInstance(o, g_ndarray) != 1) {
        PyErr_Clear();
        return 0;
    }
    if (PyObject_GetBuffer(o, v, PyBUF_C_CONTIGUOUS | PyBUF_FORMAT) != 0) {
        PyErr_Clear();
        return 0;
    }
    if (v->ndim != ndim || v->itemsize != 4 || !v->format || v->format[0] != fmt || v->format[1] != '\0') {
        PyBuffer_Release(v);
        return 0;
    }
    return 1;
}

/* An int32 scalar (not a float); 0 when it is anything else. */
static int as_i32(PyObject *o, int32_t *out)
{
    if (PyFloat_Check(o) || PyObject_IsInstance(o, g_floating) == 1)
        return 0;
    PyObject *ix = PyNumber_Index(o);
    if (!ix) {
        PyErr_Clear();
        return 0;
    }
    int overflow = 0;
    const long long v = PyLong_AsLongLongAndOverflow(ix, &overflow);
    Py_DECREF(ix);
    if (overflow || v < INT32_MIN || v > INT32_MAX || (v == -1 && PyErr_Occurred())) {
        PyErr_Clear();
        return 0;
    }
    *out = (int32_t)v;
    return 1;
}

/* A float32 scalar as numpy.float32(float(o)) gives it. */
static int as_f32(PyObject *o, float *out)
{
    if (o == Py_None)
        return 0;
    const double d = PyFloat_AsDouble(o);
    if (d == -1.0 && PyErr_Occurred()) {
        PyErr_Clear();
        return 0;
    }
    *out = (float)d;
    return 1;
}

static PyObject *zeros3(int32_t a, int32_t b, int32_t c)
{
    PyObject *shape = Py_BuildValue("(iii)", a, b, c);
    if (!shape)
        return NULL;
    PyObject *r = PyObject_CallFunctionObjArgs(g_zeros, shape, g_float32, NULL);
    Py_DECREF(shape);
    return r;
}

enum { B_IDX, B_BOX, B_BASIS, B_MOL, B_EL, B_HI, B_HE, B_N };

static void release(Py_buffer *b, const int *held)
{
    for (int k = 0; k < B_N; ++k)
        if (held[k])
            PyBuffer_Release(&b[k]);
}

/* Two zeroed float32 (ne, ne, hs) arrays and their buffers; 0 on failure
 * (with a Python error set when allocation itself failed). */
static int outputs(int32_t ne, int32_t hs, PyObject **hi, PyObject **he, Py_buffer *b, int *held)
{
    *hi = zeros3(ne, ne, hs);
    *he = *hi ? zeros3(ne, ne, hs) : NULL;
    if (*he && (held[B_HI] = take(*hi, &b[B_HI], 'f', 3)) && (held[B_HE] = take(*he, &b[B_HE], 'f', 3)))
        return 1;
    Py_XDECREF(*hi);
    Py_XDECREF(*he);
    *hi = *he = NULL;
    return 0;
}

/* multiple(indexes, boxCoords, basis, isPBC, moleculeIndex, elementIndex,
 *          numberOfElements, minDistance, maxDistance, bin, histSize,
 *          allAtoms, ncores) -> (hintra, hinter) | status | None */
static PyObject *fast_multiple(PyObject *self, PyObject *args)
{
    PyObject *o[13];
    if (!PyArg_UnpackTuple(args, "multiple", 13, 13, &o[0], &o[1], &o[2], &o[3], &o[4], &o[5], &o[6], &o[7], &o[8],
                           &o[9], &o[10], &o[11], &o[12]))
        return NULL;
    Py_buffer b[B_N];
    int held[B_N] = {0};
    int32_t ne = 0, hs = 0, nc = 0;
    float mn = 0.f, mx = 0.f, bw = 0.f;
    int ok = (held[B_IDX] = take(o[0], &b[B_IDX], 'i', 1)) && (held[B_BOX] = take(o[1], &b[B_BOX], 'f', 2)) &&
             (held[B_BASIS] = take(o[2], &b[B_BASIS], 'f', 2)) && (held[B_MOL] = take(o[4], &b[B_MOL], 'i', 1)) &&
             (held[B_EL] = take(o[5], &b[B_EL], 'i', 1)) && as_i32(o[6], &ne) && as_f32(o[7], &mn) &&
             as_f32(o[8], &mx) && as_f32(o[9], &bw) && as_i32(o[10], &hs) && as_i32(o[12], &nc) && ne >= 0 &&
             hs >= 0;
    const int isPBC = ok ? PyObject_IsTrue(o[3]) : 0;
    const int allAtoms = ok ? PyObject_IsTrue(o[11]) : 0;
    if (ok && (isPBC < 0 || allAtoms < 0)) {
        PyErr_Clear();
        ok = 0;
    }
    const Py_ssize_t n = ok ? b[B_BOX].shape[0] : 0;
    if (ok && (b[B_BOX].shape[1] != 3 || b[B_BASIS].shape[0] * b[B_BASIS].shape[1] < 9 || b[B_MOL].shape[0] < n ||
               b[B_EL].shape[0] < n))
        ok = 0;
    PyObject *hi = NULL, *he = NULL;
    if (!ok || !outputs(ne, hs, &hi, &he, b, held)) {
        release(b, held);
        if (PyErr_Occurred())
            return NULL;
        Py_RETURN_NONE;
    }
    const Py_ssize_t K = b[B_IDX].shape[0];
    int rc = 0;
    if (K > 0 && n > 0 && (int64_t)ne * ne * hs > 0) {
        Py_BEGIN_ALLOW_THREADS
        rc = frmc_multiple_pairs_histograms_coords((const int32_t *)b[B_IDX].buf, K, (const float *)b[B_BOX].buf, n,
                                                   (const float *)b[B_BASIS].buf, isPBC, (const int32_t *)b[B_MOL].buf,
                                                   (const int32_t *)b[B_EL].buf, ne, mn, mx, bw, hs, allAtoms,
                                                   (float *)b[B_HI].buf, (float *)b[B_HE].buf);
        Py_END_ALLOW_THREADS
    }
    release(b, held);
    if (rc) {
        Py_DECREF(hi);
        Py_DECREF(he);
        return PyLong_FromLong(rc);
    }
    return Py_BuildValue("(NN)", hi, he);
}

/* full(boxCoords, basis, isPBC, moleculeIndex, elementIndex, numberOfElements,
 *      minDistance, maxDistance, bin, histSize, ncores) -> (hintra, hinter) | status | None */
static PyObject *fast_full(PyObject *self, PyObject *args)
{
    PyObject *o[11];
    if (!PyArg_UnpackTuple(args, "full", 11, 11, &o[0], &o[1], &o[2], &o[3], &o[4], &o[5], &o[6], &o[7], &o[8],
                           &o[9], &o[10]))
        return NULL;
    Py_buffer b[B_N];
    int held[B_N] = {0};
    int32_t ne = 0, hs = 0, nc = 0;
    float mn = 0.f, mx = 0.f, bw = 0.f;
    int ok = (held[B_BOX] = take(o[0], &b[B_BOX], 'f', 2)) && (held[B_BASIS] = take(o[1], &b[B_BASIS], 'f', 2)) &&
             (held[B_MOL] = take(o[3], &b[B_MOL], 'i', 1)) && (held[B_EL] = take(o[4], &b[B_EL], 'i', 1)) &&
             as_i32(o[5], &ne) && as_f32(o[6], &mn) && as_f32(o[7], &mx) && as_f32(o[8], &bw) &&
             as_i32(o[9], &hs) && as_i32(o[10], &nc) && ne >= 0 && hs >= 0;
    const int isPBC = ok ? PyObject_IsTrue(o[2]) : 0;
    if (ok && isPBC < 0) {
        PyErr_Clear();
        ok = 0;
    }
    const Py_ssize_t n = ok ? b[B_BOX].shape[0] : 0;
    if (ok && (b[B_BOX].shape[1] != 3 || b[B_BASIS].shape[0] * b[B_BASIS].shape[1] < 9 || b[B_MOL].shape[0] < n ||
               b[B_EL].shape[0] < n))
        ok = 0;
    PyObject *hi = NULL, *he = NULL;
    if (!ok || !outputs(ne, hs, &hi, &he, b, held)) {
        release(b, held);
        if (PyErr_Occurred())
            return NULL;
        Py_RETURN_NONE;
    }
    int rc = 0;
    if (n >= 2 && (int64_t)ne * ne * hs > 0) {
        Py_BEGIN_ALLOW_THREADS
        rc = frmc_full_pairs_histograms_coords((const float *)b[B_BOX].buf, n, (const float *)b[B_BASIS].buf, isPBC,
                                               (const int32_t *)b[B_MOL].buf, (const int32_t *)b[B_EL].buf, ne, mn, mx,
                                               bw, hs, (float *)b[B_HI].buf, (float *)b[B_HE].buf);
        Py_END_ALLOW_THREADS
    }
    release(b, held);
    if (rc) {
        Py_DECREF(hi);
        Py_DECREF(he);
        return PyLong_FromLong(rc);
    }
    return Py_BuildValue("(NN)", hi, he);
}

/* transform(transMatrix, coords) -> (n, 3) float32 array | status | None */
static PyObject *fast_transform(PyObject *self, PyObject *args)
{
    PyObject *m, *c;
    if (!PyArg_UnpackTuple(args, "transform", 2, 2, &m, &c))
        return NULL;
    Py_buffer bm, bc, bo;
    const int hm = take(m, &bm, 'f', 2), hc = hm ? take(c, &bc, 'f', 2) : 0;
    if (!hm || !hc || bm.shape[0] * bm.shape[1] < 9 || bc.shape[1] != 3) {
        if (hm)
            PyBuffer_Release(&bm);
        if (hc)
            PyBuffer_Release(&bc);
        Py_RETURN_NONE;
    }
    const Py_ssize_t n = bc.shape[0];
    PyObject *shape = Py_BuildValue("(ni)", n, 3);
    PyObject *out = shape ? PyObject_CallFunctionObjArgs(g_zeros, shape, g_float32, NULL) : NULL;
    Py_XDECREF(shape);
    if (!out || !take(out, &bo, 'f', 2)) {
        PyBuffer_Release(&bm);
        PyBuffer_Release(&bc);
        Py_XDECREF(out);
        if (PyErr_Occurred())
            return NULL;
        Py_RETURN_NONE;
    }
    int rc = 0;
    if (n > 0) {
        Py_BEGIN_ALLOW_THREADS
        rc = frmc_transform_coordinates((const float *)bm.buf, (const float *)bc.buf, n, (float *)bo.buf);
        Py_END_ALLOW_THREADS
    }
    PyBuffer_Release(&bm);
    PyBuffer_Release(&bc);
    PyBuffer_Release(&bo);
    if (rc) {
        Py_DECREF(out);
        return PyLong_FromLong(rc);
    }
    return out;
}

static PyMethodDef kMethods[] = {
    {"multiple", fast_multiple, METH_VARARGS, "multiple_pairs_histograms_coords fast path"},
    {"full", fast_full, METH_VARARGS, "full_pairs_histograms_coords fast path"},
    {"transform", fast_transform, METH_VARARGS, "transform_coordinates fast path"},
    {NULL, NULL, 0, NULL},
};

static struct PyModuleDef kModule = {PyModuleDef_HEAD_INIT, "_fastcall", NULL, -1, kMethods};

PyMODINIT_FUNC PyInit__fastcall(void)
{
    PyObject *np = PyImport_ImportModule("numpy");
    if (!np)
        return NULL;
    g_ndarray = PyObject_GetAttrString(np, "ndarray");
    g_floating = PyObject_GetAttrString(np, "floating");
    g_zeros = PyObject_GetAttrString(np, "zeros");
    g_float32 = PyObject_GetAttrString(np, "float32");
    Py_DECREF(np);
    if (!g_ndarray || !g_floating || !g_zeros || !g_float32)
        return NULL;
    return PyModule_Create(&kModule);
}
