"""Writes tests/golden/known_answers.json: the operator known answers that the
reference's own unit tests assert, transcribed with their file:line.

Inputs are the reference's univariate seeds: a = (val, grad, hess) of
x^2 + x + 2 at x = 1, i.e. (4, 3, 2), b = (0, 1, 4), and the few other seeds
those tests use.  Op codes are those of tad_debug_scalar_op (include/tad.h)
and oracle_scalar_op.  Run: python tests/golden/make_known_answers.py
"""
import json
import math
import os

A = [4.0, 3.0, 2.0]
B = [0.0, 1.0, 4.0]
Z = [0.0, 0.0, 0.0]
H = [0.5, 3.0, 2.0]

cases = [
    # (name, op, a, b, expected (val, grad, hess), tol, source)
    ("neg", 0, A, Z, [-4.0, -3.0, -2.0], 1e-12, "tests/ScalarTestUnaryOperators.cc:12-24"),
    ("sqrt", 1, A, Z, [2.0, 3.0 / 4.0, 7.0 / 32.0], 1e-12, "tests/ScalarTestUnaryOperators.cc:39-52"),
    ("fabs+", 16, [1.0, 3.0, 6.0], Z, [1.0, 3.0, 6.0], 1e-12, "tests/ScalarTestUnaryOperators.cc:118-125"),
    ("fabs-", 16, [-1.0, 3.0, -6.0], Z, [1.0, -3.0, 6.0], 1e-12, "tests/ScalarTestUnaryOperators.cc:130-137"),
    ("exp", 5, A, Z, [math.exp(4), 3 * math.exp(4), 11 * math.exp(4)], 1e-9, "tests/ScalarTestUnaryOperators.cc:199-205"),
    ("log", 6, A, Z, [2 * math.log(2), 0.75, -1.0 / 16.0], 1e-12, "tests/ScalarTestUnaryOperators.cc:226-232"),
    ("log2", 24, A, Z, [2.0, 0.75 / math.log(2), -1.0 / 16.0 / math.log(2)], 1e-12, "tests/ScalarTestUnaryOperators.cc:253-259"),
    ("log10", 25, A, Z, [math.log10(4), 0.75 / math.log(10), -1.0 / 16.0 / math.log(10)], 1e-12,
     "tests/ScalarTestUnaryOperators.cc:280-286"),
    ("sin", 7, A, Z, [math.sin(4), 3 * math.cos(4), 2 * math.cos(4) - 9 * math.sin(4)], 1e-12,
     "tests/ScalarTestUnaryOperators.cc:307-313"),
    ("cos", 8, A, Z, [math.cos(4), -3 * math.sin(4), -2 * math.sin(4) - 9 * math.cos(4)], 1e-12,
     "tests/ScalarTestUnaryOperators.cc:334-340"),
    ("tan", 9, A, Z, [math.tan(4), 3 / math.cos(4) ** 2, 4 * (1 + 9 * math.tan(4)) / (1 + math.cos(8))], 1e-9,
     "tests/ScalarTestUnaryOperators.cc:361-367"),
    ("asin", 10, H, Z, [math.asin(0.5), 3.4641, 9.2376], 1e-4, "tests/ScalarTestUnaryOperators.cc:388-394"),
    ("acos", 11, H, Z, [math.acos(0.5), -3.4641, -9.2376], 1e-4, "tests/ScalarTestUnaryOperators.cc:415-421"),
    ("atan", 12, H, Z, [math.atan(0.5), 2.4, -4.16], 1e-12, "tests/ScalarTestUnaryOperators.cc:442-448"),
    ("sinh", 13, A, Z, [math.sinh(4), 3 * math.cosh(4), 9 * math.sinh(4) + 2 * math.cosh(4)], 1e-9,
     "tests/ScalarTestUnaryOperators.cc:469-475"),
    ("cosh", 14, A, Z, [math.cosh(4), 3 * math.sinh(4), 2 * math.sinh(4) + 9 * math.cosh(4)], 1e-9,
     "tests/ScalarTestUnaryOperators.cc:496-502"),
    ("tanh", 15, A, Z, [math.tanh(4), 3 / math.cosh(4) ** 2,
                        2 * (1 - 9 * math.sinh(4) / math.cosh(4)) / math.cosh(4) ** 2], 1e-12,
     "tests/ScalarTestUnaryOperators.cc:523-529"),
    ("asinh", 26, H, Z, [math.asinh(0.5), 2.68328, -1.43108], 1e-5, "tests/ScalarTestUnaryOperators.cc:550-556"),
    ("acosh", 27, A, Z, [math.acosh(4), math.sqrt(3 / 5), -2 / 5 / math.sqrt(15)], 1e-12,
     "tests/ScalarTestUnaryOperators.cc:577-583"),
    ("atanh", 28, H, Z, [math.atanh(0.5), 4.0, 18.6667], 1e-4, "tests/ScalarTestUnaryOperators.cc:604-610"),
    ("pow_int3", 3, A, [3.0, 0.0, 0.0], [64.0, 144.0, 312.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:38-47"),
    ("pow_int0", 3, A, [0.0, 0.0, 0.0], [1.0, 0.0, 0.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:17-26"),
    ("pow_int1", 3, A, [1.0, 0.0, 0.0], [4.0, 3.0, 2.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:28-36"),
    ("pow_real1.5", 4, A, [1.5, 0.0, 0.0], [8.0, 9.0, 75.0 / 8.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:67-75"),
    ("pow_real3", 4, A, [3.0, 0.0, 0.0], [64.0, 144.0, 312.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:97-105"),
    ("plus", 17, A, B, [4.0, 4.0, 6.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:128-137"),
    ("plus_passive", 29, A, [1.0, 0.0, 0.0], [5.0, 3.0, 2.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:141-149"),
    ("minus", 18, A, B, [4.0, 2.0, -2.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:204-213"),
    ("passive_minus", 31, A, [1.0, 0.0, 0.0], [-3.0, -3.0, -2.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:227-236"),
    ("mult", 19, A, B, [0.0, 4.0, 22.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:280-289"),
    ("mult_passive", 30, A, [2.0, 0.0, 0.0], [8.0, 6.0, 4.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:291-300"),
    ("div", 20, [1.0, 1.0, 4.0], A, [0.25, 1.0 / 16.0, 25.0 / 32.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:356-365"),
    ("div_passive", 32, [1.0, 1.0, 4.0], [2.0, 0.0, 0.0], [0.5, 0.5, 2.0], 1e-12, "tests/ScalarTestBinaryOperators.cc:370-378"),
]

out = [dict(name=n, op=op, a=a, b=b, expected=e, tol=t, source=s) for (n, op, a, b, e, t, s) in cases]
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
with open(path, "w") as f:
    json.dump(out, f, indent=1)
print(path, len(out))
