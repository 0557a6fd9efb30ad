"""Host-side pieces of the CPU reference recipe (no reference needed)."""
from oracle.refbuild import rewrite_get


def test_rewrite_get_member_calls():
    cases = {
        "a.get<0>()": "thrust::get<0>(a)",
        "x = tup.get<0>().get<1>();": "x = thrust::get<1>(thrust::get<0>(tup));",
        "normal.get<2>() = v;": "thrust::get<2>(normal) = v;",
        "f(it.get_iterator_tuple().get<1>())": "f(thrust::get<1>(it.get_iterator_tuple()))",
        "p->q.get<3>()": "thrust::get<3>(p->q)",
        "s[i].get<0>()": "thrust::get<0>(s[i])",
        "a.get<0>() + b.get<1>()": "thrust::get<0>(a) + thrust::get<1>(b)",
    }
    for src, want in cases.items():
        assert rewrite_get(src) == want, src


def test_rewrite_get_leaves_other_code():
    s = "auto p = ptr.get(); int y = 1.5f * z; thrust::get<0>(t);"
    assert rewrite_get(s) == s
